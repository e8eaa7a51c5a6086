"""Python front of the CPU FP64 oracle (``sgdg_oracle.c``).

TEST INFRASTRUCTURE ONLY: the parity oracle and the timed CPU baseline.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs import it;
the product package never does.

Function names follow the reference (GalerkinSparseGrids.jl) so the tests read
like ``test/*.jl``.  Matrices come back as ``scipy.sparse.csc_matrix`` with the
reference's stored pattern (numerical zeros kept where Julia keeps them).
"""
import ctypes
import os
import subprocess

import numpy as np
import scipy.sparse as sp

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "build", "liboracle.so")
SCHEMES = {"sparse": 0, "full": 1}

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(force=False):
    """Compile the oracle with gcc (no FMA contraction, OpenMP for the baseline)."""
    src = os.path.join(_HERE, "sgdg_oracle.c")
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(src):
        return _SO
    os.makedirs(os.path.dirname(_SO), exist_ok=True)
    tmp = _SO + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-fopenmp",
                           "-ffp-contract=off", "-o", tmp, src, "-lm"])
    os.replace(tmp, _SO)
    return _SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        vp = ctypes.c_void_p
        L.or_init.restype = ctypes.c_int
        L.or_dg_coeffs.argtypes = [ctypes.c_int, _f64p]
        L.or_leg_coeffs.argtypes = [_f64p]
        L.or_v.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double]
        L.or_v.restype = ctypes.c_double
        L.or_basis.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double]
        L.or_basis.restype = ctypes.c_double
        for name, args in [("or_hier2pos", [ctypes.c_int] * 2), ("or_pos_dlf", [ctypes.c_int] * 2),
                           ("or_dmat1d", [ctypes.c_int] * 2), ("or_dmatrix", [ctypes.c_int] * 5),
                           ("or_laplacian", [ctypes.c_int] * 4), ("or_wave_rhs", [vp]), ("or_matmul", [vp, vp]),
                           ("or_advection", [ctypes.c_int] * 4 + [_f64p]),
                           ("or_from_csc", [ctypes.c_int64] * 3 + [_i64p, _i32p, _f64p])]:
            f = getattr(L, name)
            f.argtypes = args
            f.restype = vp
        L.or_mat_free.argtypes = [vp]
        L.or_mat_info.argtypes = [vp] + [ctypes.POINTER(ctypes.c_int64)] * 3
        L.or_mat_export_csc.argtypes = [vp, _i64p, _i32p, _f64p]
        L.or_mat_export_csr.argtypes = [vp, _i64p, _i32p, _f64p]
        L.or_get_size.argtypes = [ctypes.c_int] * 4
        L.or_get_size.restype = ctypes.c_int64
        L.or_index_map.argtypes = [ctypes.c_int] * 4 + [_i32p] * 3
        L.or_spmv_csc.argtypes = [vp, _f64p, _f64p]
        L.or_csr_from_mat.argtypes = [vp]
        L.or_csr_from_mat.restype = vp
        L.or_csr_free.argtypes = [vp]
        L.or_csr_spmv.argtypes = [vp, _f64p, _f64p, ctypes.c_int]
        L.or_rk4_csr.argtypes = [vp, _f64p, ctypes.c_double, ctypes.c_int64, ctypes.c_int]
        L.or_max_threads.restype = ctypes.c_int
        L.or_fourier_coeffs.argtypes = [ctypes.c_int] * 5 + [_i32p, _f64p, _i32p, _f64p, _f64p]
        L.or_tensor_construct.argtypes = [ctypes.c_int] * 4 + [_f64p, _f64p]
        L.or_reconstruct.argtypes = [ctypes.c_int] * 4 + [_f64p, ctypes.c_int64, _f64p, _f64p]
        L.or_transform_1d.argtypes = [ctypes.c_int] * 3
        L.or_transform_1d.restype = vp
        L.or_transform.argtypes = [ctypes.c_int] * 4 + [vp]
        L.or_transform.restype = vp
        L.or_cell_index.argtypes = [ctypes.c_double, ctypes.c_int]
        L.or_cell_index.restype = ctypes.c_int
        L.or_init()
        _lib = L
    return _lib


class _Mat:
    """Owns an ``or_mat*`` from the C oracle."""

    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        if self.ptr and _lib is not None:
            _lib.or_mat_free(self.ptr)
            self.ptr = None

    def info(self):
        m, n, z = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        lib().or_mat_info(self.ptr, ctypes.byref(m), ctypes.byref(n), ctypes.byref(z))
        return m.value, n.value, z.value

    def csc(self):
        m, n, z = self.info()
        cp = np.zeros(n + 1, np.int64)
        rv = np.zeros(max(z, 1), np.int32)
        nv = np.zeros(max(z, 1), np.float64)
        lib().or_mat_export_csc(self.ptr, cp, rv, nv)
        return sp.csc_matrix((nv[:z], rv[:z], cp), shape=(m, n))

    def csr_arrays(self):
        m, n, z = self.info()
        rp = np.zeros(m + 1, np.int64)
        col = np.zeros(max(z, 1), np.int32)
        val = np.zeros(max(z, 1), np.float64)
        lib().or_mat_export_csr(self.ptr, rp, col, val)
        return rp, col[:z], val[:z]


def _scheme(scheme):
    if scheme not in SCHEMES:
        raise ValueError("scheme must be 'sparse' or 'full'")
    return SCHEMES[scheme]


# --- basis (src/dg_basis.jl, src/1d_dg_functions.jl) -------------------------
def dg_coeffs(k):
    """dg_coeffs[k] as a (2k, k) array: column = mode (src/1d_dg_functions.jl:52-62)."""
    out = np.zeros(2 * k * k)
    lib().or_dg_coeffs(k, out)
    return out.reshape(k, 2 * k).T.copy()


def leg_coeffs():
    out = np.zeros(11 * 22)
    lib().or_leg_coeffs(out)
    return out.reshape(11, 22)


def v(k, level, cell, mode, x):
    return lib().or_v(k, level, cell, mode, float(x))


def basis(level, cell, mode, x):
    return lib().or_basis(level, cell, mode, float(x))


# --- index map (src/dg_vmethods.jl) ------------------------------------------
def get_size(D, k, n, scheme="sparse"):
    return int(lib().or_get_size(D, k, n, _scheme(scheme)))


def index_map(D, k, n, scheme="sparse"):
    """V2Dref as three (N, D) int32 arrays of 1-based level, cell, mode."""
    N = get_size(D, k, n, scheme)
    L = np.zeros(N * D, np.int32)
    C = np.zeros(N * D, np.int32)
    M = np.zeros(N * D, np.int32)
    lib().or_index_map(D, k, n, _scheme(scheme), L, C, M)
    return L.reshape(N, D), C.reshape(N, D), M.reshape(N, D)


# --- operators ----------------------------------------------------------------
def hier2pos(k, n):
    return _Mat(lib().or_hier2pos(k, n)).csc()


def periodic_pos_DLF_matrix(k, n):
    return _Mat(lib().or_pos_dlf(k, n)).csc()


def periodic_DLF_matrix(k, n):
    """1D hierarchical periodic DG derivative (src/1d_derivative.jl:113-117)."""
    return _Mat(lib().or_dmat1d(k, n)).csc()


def pos_wave_rhs_raw(k, n):
    """wave_evolve_1D's right-hand side in the position basis
    (src/pdes.jl:89-121, basis = "pos"): wave_data(D_op * D_op), D_op =
    periodic_pos_DLF_matrix.  Returns (D_op, laplac, RHS) as oracle matrices."""
    A = _Mat(lib().or_pos_dlf(k, n))
    lap = _Mat(lib().or_matmul(A.ptr, A.ptr))
    return A, lap, _Mat(lib().or_wave_rhs(lap.ptr))


def D_matrix(D, d, k, n, scheme="sparse"):
    """D-dim derivative along dim d, 1-based (src/multidim_derivative.jl:61-65)."""
    return _Mat(lib().or_dmatrix(D, d, k, n, _scheme(scheme))).csc()


def D_matrix_raw(D, d, k, n, scheme="sparse"):
    return _Mat(lib().or_dmatrix(D, d, k, n, _scheme(scheme)))


def grad_matrix(D, k, n, scheme="sparse"):
    return [D_matrix(D, d, k, n, scheme) for d in range(1, D + 1)]


def laplacian_matrix_raw(D, k, n, scheme="sparse"):
    return _Mat(lib().or_laplacian(D, k, n, _scheme(scheme)))


def laplacian_matrix(D, k, n, scheme="sparse"):
    return laplacian_matrix_raw(D, k, n, scheme).csc()


def wave_rhs_raw(D, k, n, scheme="sparse"):
    lap = laplacian_matrix_raw(D, k, n, scheme)
    return _Mat(lib().or_wave_rhs(lap.ptr))


def advection_matrix_raw(D, k, n, a, scheme="sparse"):
    a = np.ascontiguousarray(a, np.float64)
    assert a.shape == (D,)
    return _Mat(lib().or_advection(D, k, n, _scheme(scheme), a))


def from_csc(A):
    A = sp.csc_matrix(A)
    A.sort_indices()
    return _Mat(lib().or_from_csc(A.shape[0], A.shape[1], A.nnz, np.ascontiguousarray(A.indptr, np.int64),
                                  np.ascontiguousarray(A.indices, np.int32),
                                  np.ascontiguousarray(A.data, np.float64)))


class CSR:
    """Row-parallel CSR copy of an oracle matrix, for the timed CPU baseline."""

    def __init__(self, mat):
        self.mat = mat
        self.ptr = lib().or_csr_from_mat(mat.ptr)
        self.m = mat.info()[0]

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.or_csr_free(self.ptr)
            self.ptr = None

    def spmv(self, x, nthreads=1):
        y = np.zeros(self.m)
        lib().or_csr_spmv(self.ptr, np.ascontiguousarray(x, np.float64), y, nthreads)
        return y

    def rk4(self, y0, dt, nsteps, nthreads=1):
        y = np.array(y0, np.float64, copy=True)
        lib().or_rk4_csr(self.ptr, y, float(dt), int(nsteps), int(nthreads))
        return y


def spmv_csc(mat, x):
    m = mat.info()[0]
    y = np.zeros(m)
    lib().or_spmv_csc(mat.ptr, np.ascontiguousarray(x, np.float64), y)
    return y


def max_threads():
    return int(lib().or_max_threads())


# --- projection / reconstruction ---------------------------------------------
def fourier_coeffs(D, k, n, modes, scheme="sparse"):
    """Coefficients of sum_m amp*trig(2*pi*a.x + phase).

    ``modes`` is a list of (a (D ints), amp, kind, phase) with kind 'sin'/'cos'.
    """
    N = get_size(D, k, n, scheme)
    nm = len(modes)
    avec = np.zeros(nm * D, np.int32)
    amp = np.zeros(nm)
    kind = np.zeros(nm, np.int32)
    phase = np.zeros(nm)
    for i, (a, am, kd, ph) in enumerate(modes):
        avec[i * D:(i + 1) * D] = a
        amp[i] = am
        kind[i] = 1 if kd == "cos" else 0
        phase[i] = ph
    out = np.zeros(N)
    lib().or_fourier_coeffs(D, k, n, _scheme(scheme), nm, avec, amp, kind, phase, out)
    return out


def tensor_construct(D, k, n, coeffs1d, scheme="sparse"):
    c = np.ascontiguousarray(np.stack([np.asarray(v, np.float64) for v in coeffs1d]).ravel())
    out = np.zeros(get_size(D, k, n, scheme))
    lib().or_tensor_construct(D, k, n, _scheme(scheme), c, out)
    return out


def cell_index(x, l):
    return int(lib().or_cell_index(float(x), int(l)))


def reconstruct(D, k, n, coeffs, pts, scheme="sparse"):
    pts = np.ascontiguousarray(np.atleast_2d(pts), np.float64)
    out = np.zeros(pts.shape[0])
    lib().or_reconstruct(D, k, n, _scheme(scheme), np.ascontiguousarray(coeffs, np.float64), pts.shape[0],
                         pts, out)
    return out


def vcoeffs_1d(k, n, f, q=24):
    """1D hierarchical coefficients of a vectorised f by Gauss-Legendre per
    polynomial piece (the oracle's stand-in for hquadrature, dg_vmethods.jl:149-179)."""
    gx, gw = np.polynomial.legendre.leggauss(q)
    out = []
    for L in range(1, n + 2):
        lvl = L - 1
        nc = 1 << max(0, L - 2)
        w = 1.0 / (1 << max(0, lvl - 1))
        for c in range(1, nc + 1):
            x0, x1 = (c - 1) * w, c * w
            halves = 1 if lvl == 0 else 2
            for m in range(1, k + 1):
                s = 0.0
                for hf in range(halves):
                    a0 = x0 + hf * (x1 - x0) / halves
                    a1 = x0 + (hf + 1) * (x1 - x0) / halves
                    xs = 0.5 * (a0 + a1) + 0.5 * (a1 - a0) * gx
                    vv = np.array([v(k, lvl, c, m, x) for x in xs])
                    s += float(np.sum(gw * vv * f(xs))) * 0.5 * (a1 - a0)
                out.append(s)
    return np.array(out)


def pos_vcoeffs_1d(k, level, f, q=24):
    """pos_vcoeffs_DG (src/1d_dg_functions.jl:103-117): the integral of
    basis(level, cell, mode) * f over each cell (mode fastest), by q-point
    Gauss-Legendre per cell (the oracle's stand-in for hquadrature)."""
    gx, gw = np.polynomial.legendre.leggauss(q)
    h = 1.0 / (1 << level)
    out = []
    for c in range(1, (1 << level) + 1):
        xs = (c - 1) * h + 0.5 * h * (1 + gx)
        fx = f(xs)
        for m in range(1, k + 1):
            bb = np.array([basis(level, c, m, x) for x in xs])
            out.append(float(np.sum(gw * bb * fx)) * 0.5 * h)
    return np.array(out)


def energy(D, k, n, state, scheme="sparse", grads=None):
    """energy_func for one stored state (src/pdes.jl:258-273)."""
    N = get_size(D, k, n, scheme)
    grads = grads if grads is not None else grad_matrix(D, k, n, scheme)
    u, ut = state[:N], state[N:]
    return sum(float(np.sum((G @ u) ** 2)) for G in grads) + float(np.sum(ut ** 2))


# ------------------------------------------------------- nodal transforms ----
TRANSFORMS = {("modal", "nodal"): 0, ("nodal", "points"): 1, ("points", "nodal"): 2, ("nodal", "modal"): 3}


def transform_1D(k, n, frm, to):
    """transform_1D (src/1d_nodal_basis.jl:350-414) for the four maps of the
    Vlasov evolver, CSC."""
    return _Mat(lib().or_transform_1d(k, n, TRANSFORMS[(frm, to)])).csc()


def transform(D, k, n, frm, to, scheme="sparse"):
    """transform(D, k, n, from, to) (src/multidim_nodal_basis.jl:83-124),
    assembled like the reference (restricted Kronecker product), CSC."""
    T1 = _Mat(lib().or_transform_1d(k, n, TRANSFORMS[(frm, to)]))
    return _Mat(lib().or_transform(D, k, n, _scheme(scheme), T1.ptr)).csc()


def get_one_modal(D, k, n, scheme="sparse"):
    """src/basic_function_exact_coeffs.jl:5-8"""
    out = np.zeros(get_size(D, k, n, scheme))
    out[0] = 1.0
    return out


def get_xi_modal(D, i, k, n, scheme="sparse"):
    """src/basic_function_exact_coeffs.jl:11-17: coefficients of 2 x_i - 1."""
    one = np.zeros(k << n)
    one[0] = 1.0
    xi = np.zeros(k << n)
    xi[1] = 1.0 / np.sqrt(3.0)
    return tensor_construct(D, k, n, [xi if d == i else one for d in range(1, D + 1)], scheme)


def vlasov_rhs(D, k, n, ops, F_point, f):
    """steprule of vlasov_evolve (src/pdes.jl:174-192) with assembled
    operators ``ops`` = (Ds (2D CSR), m2n, n2p, p2n, n2m) and the velocity
    points v_point built as in src/pdes.jl:166-172."""
    Ds, m2n, n2p, p2n, n2m, v_point = ops
    # the 2D derivatives go through m2n and n2p as the columns of one block
    # (scipy sums each column's row in the same order as a single SpMV, so
    # the values are those of separate products; the matrix is read once)
    grads = np.column_stack([Ds[d] @ f for d in range(2 * D)])
    pts = n2p @ (m2n @ grads)
    xpt = [pts[:, d] for d in range(D)]
    ppt = [pts[:, D + d] for d in range(D)]
    c1 = sum(v_point[d] * xpt[d] for d in range(D))
    c2 = sum(F_point[d] * ppt[d] for d in range(D))
    return n2m @ (p2n @ (-c1 + c2))


def vlasov_operators(D, k, n, scheme="sparse"):
    """Assembled operators of vlasov_evolve for D space dimensions (2D-dim
    phase space): grad_matrix(2D), the four transforms and v_point."""
    P = 2 * D
    Ds = [D_matrix(P, d, k, n, scheme).tocsr() for d in range(1, P + 1)]
    m2n = transform(P, k, n, "modal", "nodal", scheme).tocsr()
    n2p = transform(P, k, n, "nodal", "points", scheme).tocsr()
    p2n = transform(P, k, n, "points", "nodal", scheme).tocsr()
    n2m = transform(P, k, n, "nodal", "modal", scheme).tocsr()
    v_point = [n2p @ (m2n @ get_xi_modal(P, D + d, k, n, scheme)) for d in range(1, D + 1)]
    return Ds, m2n, n2p, p2n, n2m, v_point


def vlasov_rk4(D, k, n, ops, F_point, f0, dt, nsteps):
    """Classical RK4 on the Vlasov right-hand side (FP64)."""
    y = np.array(f0, np.float64)
    for _ in range(nsteps):
        k1 = vlasov_rhs(D, k, n, ops, F_point, y)
        k2 = vlasov_rhs(D, k, n, ops, F_point, y + 0.5 * dt * k1)
        k3 = vlasov_rhs(D, k, n, ops, F_point, y + 0.5 * dt * k2)
        k4 = vlasov_rhs(D, k, n, ops, F_point, y + dt * k3)
        y = y + (dt / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4)
    return y
