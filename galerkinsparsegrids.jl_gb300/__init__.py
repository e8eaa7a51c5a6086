"""GalerkinSparseGrids.jl's derivative-operator / RK time-stepping path on one
GB300, behind the reference's API.

Names, argument meaning and errors follow src/GalerkinSparseGrids.jl's exports
(get_size, V2Dref, D2Vref, vcoeffs_DG, tensor_construct, D_matrix,
grad_matrix, laplacian_matrix, wave_evolve) so code written against the
reference reads the same.  Coefficient vectors use the reference's layout
unchanged.  All compute runs in libsgdg.so (hand-written sm_103a CUDA); there
is no CPU fallback: without the library or a GPU every compute call raises.

Host-side helpers here (coefficient projection, index maps, sparse exports)
are set-up and I/O around the hot path, like the reference's own set-up code.
"""
import ctypes
import functools
import os

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import SGDGError, check, lib

__all__ = [
    "get_size", "index_map", "V2Dref", "D2Vref", "V2D", "D2V", "dg_coeffs", "vcoeffs_DG", "vcoeffs_1d", "pos_vcoeffs_DG",
    "tensor_construct", "fourier_coeffs", "periodic_DLF_matrix", "D_matrix", "grad_matrix", "laplacian_matrix",
    "SparseGridOperator", "wave_evolve", "advect_evolve", "energy_func", "Batch", "SGDGError", "set_hbm_budget",
    "hbm_in_use",
]


def _scheme(scheme):
    if scheme not in _lib.SCHEMES:
        raise ValueError("scheme must be \"sparse\" or \"full\"")
    return _lib.SCHEMES[scheme]


def _method(method):
    if method not in _lib.METHODS:
        raise ValueError("method must be \"plain\" or \"matfree\"")
    return _lib.METHODS[method]


# ---------------------------------------------------------------- layout ----
def get_size(D, k, n, scheme="sparse"):
    """Number of coefficients (src/dg_vmethods.jl:35-45)."""
    N = ctypes.c_int64()
    check(lib().sgdg_get_size(D, k, n, _scheme(scheme), ctypes.byref(N)))
    return N.value


def index_map(D, k, n, scheme="sparse"):
    """(level, cell, mode) of every coefficient as three (N, D) int32 arrays, 1-based."""
    N = get_size(D, k, n, scheme)
    L = np.zeros(N * D, np.int32)
    C = np.zeros(N * D, np.int32)
    M = np.zeros(N * D, np.int32)
    check(lib().sgdg_index_map(D, k, n, _scheme(scheme), L, C, M))
    return L.reshape(N, D), C.reshape(N, D), M.reshape(N, D)


def V2Dref(D, k, n, scheme="sparse"):
    """Vector of (level, cell, mode) tuples (src/dg_vmethods.jl:123-142)."""
    L, C, M = index_map(D, k, n, scheme)
    return [(tuple(L[i]), tuple(C[i]), tuple(M[i])) for i in range(L.shape[0])]


def D2Vref(D, k, n, scheme="sparse"):
    """Dict (level, cell, mode) -> 1-based vector index (src/dg_vmethods.jl:102-121)."""
    return {t: i + 1 for i, t in enumerate(V2Dref(D, k, n, scheme))}


def V2D(D, k, n, vect, scheme="sparse"):
    """Vector -> {level: {cell: {mode: value}}} (src/dg_vmethods.jl:76-100)."""
    out = {}
    for (lv, cl, md), val in zip(V2Dref(D, k, n, scheme), vect):
        out.setdefault(lv, {}).setdefault(cl, {})[md] = val
    return out


def D2V(D, k, n, coeffs, scheme="sparse"):
    """Inverse of V2D (src/dg_vmethods.jl:48-74)."""
    return np.array([coeffs[lv][cl][md] for (lv, cl, md) in V2Dref(D, k, n, scheme)])


def dg_coeffs(k):
    """dg_coeffs[k] (src/1d_dg_functions.jl:52-62) as a (2k, k) array."""
    out = np.zeros(2 * k * k)
    check(lib().sgdg_dg_coeffs(k, out))
    return out.reshape(k, 2 * k).T.copy()


# ------------------------------------------------------------ projection ----
def _legendre_monomials(m):
    """Orthonormal Legendre polynomial of degree m on [-1,1], monomial coefficients."""
    c = np.polynomial.legendre.leg2poly(np.eye(m + 1)[m])
    return c * np.sqrt((2 * m + 1) / 2.0)


def _eval_v(k, lvl, cell, mode, x):
    """Hierarchical basis function v (src/dg_methods.jl:27-36) at points x (vectorised)."""
    x = np.asarray(x, np.float64)
    if lvl == 0:
        p = _legendre_monomials(mode - 1)
        return np.sqrt(2.0) * np.polynomial.polynomial.polyval(2 * x - 1, p) * ((x >= 0) & (x <= 1))
    y = (1 << lvl) * x - (2 * cell - 1)
    c = dg_coeffs(k)[:, mode - 1]
    a, b = c[:k], c[k:]
    val = np.polynomial.polynomial.polyval(y, a) + np.sign(y) * np.polynomial.polynomial.polyval(y, b)
    return np.sqrt(float(1 << lvl)) * val * (np.abs(y) <= 1)


@functools.lru_cache(maxsize=64)
def _pieces_1d(k, n, q, hmax=1.0 / 16):
    """Per 1D block: quadrature nodes/weights on its polynomial pieces (split
    further into sub-intervals no wider than hmax) and the basis values there.
    Returns list over levels L=1..n+1 of arrays nodes (cells, P),
    weights (P,), values (cells, k, P)."""
    gx, gw = np.polynomial.legendre.leggauss(q)
    out = []
    for L in range(1, n + 2):
        lvl = L - 1
        nc = 1 << max(0, L - 2)
        w = 1.0 / (1 << max(0, lvl - 1))
        halves = 1 if lvl == 0 else 2
        sub = max(1, int(np.ceil(w / halves / hmax - 1e-12)))
        parts = halves * sub  # sub-intervals per cell, never straddling the midpoint
        loc = np.concatenate([(h + 0.5 + 0.5 * gx) / parts for h in range(parts)])  # in [0,1] of the cell
        wts = np.concatenate([0.5 * gw / parts for _ in range(parts)]) * w
        nodes = (np.arange(nc)[:, None] + loc[None, :]) * w
        vals = np.stack([np.stack([_eval_v(k, lvl, c + 1, m, nodes[c]) for m in range(1, k + 1)])
                         for c in range(nc)])
        out.append((nodes, wts, vals))
    return out


def vcoeffs_1d(k, n, f, q=None):
    """1D hierarchical coefficients of a vectorised f (1D vector order)."""
    q = q or max(8, k + 4)
    res = []
    for nodes, wts, vals in _pieces_1d(k, n, q):
        res.append(np.einsum("cmp,cp,p->cm", vals, f(nodes), wts).ravel())
    return np.concatenate(res)


def vcoeffs_DG(D, k, n, f, scheme="sparse", q=None, device=False):
    """Coefficient vector of f (src/dg_vmethods.jl:149-179).

    ``f`` takes an (npts, D) array of points and returns npts values.  The
    reference integrates each basis function with hcubature; here every level
    block is integrated at once with tensor Gauss-Legendre rules on the
    polynomial pieces (exact for polynomials of degree < 2q).  With
    ``device=True`` f is sampled on the host at every block's tensor grid of
    nodes and the GPU contracts the samples dimension by dimension
    (sgdg_vcoeffs_contract)."""
    q = q or max(6, k + 3)
    if device:
        return _vcoeffs_device(D, k, n, f, scheme, q)
    if D == 1:
        return vcoeffs_1d(k, n, lambda x: np.asarray(f(x.reshape(-1, 1)), np.float64).reshape(x.shape), q)
    pieces = _pieces_1d(k, n, q)
    L, _, _ = index_map(D, k, n, scheme)
    N = L.shape[0]
    out = np.empty(N)
    lv_rows = {}
    pos = 0
    while pos < N:
        lv = tuple(L[pos])
        cells = [1 << max(0, l - 2) for l in lv]
        size = int(np.prod(cells)) * k ** D
        lv_rows[lv] = (pos, size)
        pos += size
    for lv, (pos, size) in lv_rows.items():
        nodes = [pieces[l - 1][0] for l in lv]  # (cells_q, P_q)
        grids = np.meshgrid(*[nd.ravel() for nd in nodes], indexing="ij")
        pts = np.stack([g.ravel() for g in grids], axis=1)
        F = np.asarray(f(pts), np.float64).reshape([nd.size for nd in nodes])
        shape = []
        for nd in nodes:
            shape += [nd.shape[0], nd.shape[1]]
        F = F.reshape(shape)  # (c1, p1, c2, p2, ...)
        for qd, l in enumerate(lv):
            _, wts, vals = pieces[l - 1]
            W = vals * wts[None, None, :]  # (c, m, p)
            # contract axis pair (c_q, p_q) currently at positions (2q, 2q+1) -> (c_q, m_q)
            F = np.moveaxis(F, (2 * qd, 2 * qd + 1), (0, 1))
            F = np.einsum("cp...,cmp->cm...", F, W)
            F = np.moveaxis(F, (0, 1), (2 * qd, 2 * qd + 1))
        # axes (c1, m1, ..., cD, mD) -> reference order: cells (dim 1 fastest) then modes (dim 1 fastest)
        order = [2 * q for q in reversed(range(D))] + [2 * q + 1 for q in reversed(range(D))]
        out[pos:pos + size] = np.transpose(F, order).ravel()
    return out


def _vcoeffs_device(D, k, n, f, scheme, q):
    pieces = _pieces_1d(k, n, q)
    npts = np.array([nodes.shape[1] for nodes, _, _ in pieces], np.int32)
    wtab = np.concatenate([(vals * wts[None, None, :]).ravel() for _, wts, vals in pieces])
    L, _, _ = index_map(D, k, n, scheme)
    N = L.shape[0]
    samples = []
    pos = 0
    while pos < N:
        lv = tuple(int(v) for v in L[pos])
        nodes = [pieces[l - 1][0].ravel() for l in lv]  # dimension q: cell * P + node
        grids = np.meshgrid(*nodes[::-1], indexing="ij")  # last axis (dimension 1) fastest
        pts = np.stack([g.ravel() for g in grids[::-1]], axis=1)
        samples.append(np.asarray(f(pts), np.float64).reshape(-1))
        pos += int(np.prod([1 << max(0, l - 2) for l in lv])) * k ** D
    out = np.empty(N)
    check(lib().sgdg_vcoeffs_contract(D, k, n, _scheme(scheme), npts, np.ascontiguousarray(wtab),
                                      np.ascontiguousarray(np.concatenate(samples)), out))
    return out


def _i1d(k, L, C, M):
    start = np.where(L >= 2, 1 << np.maximum(L - 2, 0), 0)
    return k * (start + C - 1) + M - 1


def _tensor_sum(D, k, n, Z, coef, scheme):
    """sum_t amp_t part_t(e^{i phi_t} prod_d Z[t, d][i_d]) on the GPU."""
    Zc = np.ascontiguousarray(np.asarray(Z, np.complex128))
    if Zc.ndim != 3 or Zc.shape[1:] != (D, k << n):
        raise ValueError("Z must be (terms, D, k 2^n)")
    out = np.empty(get_size(D, k, n, scheme))
    c = np.ascontiguousarray(coef, np.float64)
    check(lib().sgdg_tensor_sum(D, k, n, _scheme(scheme), Zc.shape[0], Zc.view(np.float64).reshape(-1),
                                c.reshape(-1), out))
    return out


def tensor_construct(D, k, n, vcoeff_array, scheme="sparse", device=False):
    """Coefficients of prod_d f_d(x_d) from 1D coefficient vectors
    (src/tensor_construct.jl:57-63); ``device=True`` computes them on the GPU."""
    if device:
        Z = np.asarray([np.asarray(v, np.float64) for v in vcoeff_array])[None].astype(np.complex128)
        return _tensor_sum(D, k, n, Z, [[1.0, 1.0, 0.0, 0.0]], scheme)
    L, C, M = index_map(D, k, n, scheme)
    out = np.ones(L.shape[0])
    for q in range(D):
        out *= np.asarray(vcoeff_array[q], np.float64)[_i1d(k, L[:, q], C[:, q], M[:, q])]
    return out


def fourier_coeffs(D, k, n, modes, scheme="sparse", device=False):
    """Coefficients of sum_m amp * trig(2 pi a.x + phase), exactly separable:
    ``modes`` = [(a (D ints), amp, "sin"|"cos", phase), ...].  The 1D
    projections are computed on the host; ``device=True`` builds the D-dim
    vector from them on the GPU."""
    if device:
        Z = np.asarray([[_fourier_1d(k, n, int(a[q])) for q in range(D)] for a, _, _, _ in modes])
        coef = []
        for a, amp, kind, ph in modes:
            z0 = np.exp(1j * ph)
            coef.append([amp, z0.real, z0.imag, 0.0 if kind == "cos" else 1.0])
        return _tensor_sum(D, k, n, Z, coef, scheme)
    idx = _index_1d(D, k, n, scheme)
    out = np.zeros(idx[0].shape[0])
    for a, amp, kind, ph in modes:
        z = np.exp(1j * ph) * np.ones(idx[0].shape[0], complex)
        for q in range(D):
            z *= _fourier_1d(k, n, int(a[q]))[idx[q]]
        out += amp * (z.real if kind == "cos" else z.imag)
    return out


@functools.lru_cache(maxsize=16)
def _index_1d(D, k, n, scheme):
    L, C, M = index_map(D, k, n, scheme)
    return [_i1d(k, L[:, q], C[:, q], M[:, q]) for q in range(D)]


@functools.lru_cache(maxsize=256)
def _fourier_1d(k, n, a):
    """1D coefficients of exp(2 pi i a x)."""
    re = vcoeffs_1d(k, n, lambda x: np.cos(2 * np.pi * a * x), q=max(12, k + 8))
    im = vcoeffs_1d(k, n, lambda x: np.sin(2 * np.pi * a * x), q=max(12, k + 8))
    return re + 1j * im


# ------------------------------------------------------------- operators ----
def _csr_from(nnz_fn, export_fn, m):
    nnz = ctypes.c_int64()
    check(nnz_fn(ctypes.byref(nnz)))
    rp = np.zeros(m + 1, np.int64)
    col = np.zeros(max(nnz.value, 1), np.int32)
    val = np.zeros(max(nnz.value, 1), np.float64)
    check(export_fn(rp, col, val))
    return sp.csr_matrix((val[:nnz.value], col[:nnz.value], rp), shape=(m, m))


def periodic_DLF_matrix(k, n, basis="hier"):
    """1D periodic DG derivative (src/1d_derivative.jl:136-148), CSR: the
    hierarchical Q' A Q or, with basis="pos", the position-basis A =
    periodic_pos_DLF_matrix (src/1d_derivative.jl:108-111)."""
    if basis == "pos":
        return SparseGridOperator(1, k, n, basis="pos").csr(1)
    if basis != "hier":
        raise ValueError("basis must be \"hier\" or \"pos\" (nodal and point are not built)")
    L = lib()
    return _csr_from(lambda p: L.sgdg_dlf_1d_nnz(k, n, p), lambda a, b, c: L.sgdg_dlf_1d_export(k, n, a, b, c),
                     k << n)


def pos_vcoeffs_DG(k, level, f, q=None, hmax=1.0 / 16):
    """Position-basis coefficients of f (src/1d_dg_functions.jl:103-117): for
    cell = 1..2^level and mode = 1..k (mode fastest) the integral of
    basis(level, cell, mode) f over the cell, basis the orthonormal Legendre
    polynomial of the cell (src/1d_dg_functions.jl:83-93).  The reference
    integrates each with hquadrature; here every cell at once with a q-point
    Gauss-Legendre rule on sub-intervals no wider than hmax.  ``f`` takes an
    (npts, 1) array of points and returns npts values."""
    q = q or max(8, k + 4)
    gx, gw = np.polynomial.legendre.leggauss(q)
    ncell = 1 << level
    h = 1.0 / ncell
    sub = max(1, int(np.ceil(h / hmax - 1e-12)))
    loc = np.concatenate([(s + 0.5 + 0.5 * gx) / sub for s in range(sub)])  # in [0, 1] of a cell
    wts = np.concatenate([0.5 * gw / sub for _ in range(sub)]) * h
    B = np.stack([np.sqrt(2.0) * np.polynomial.polynomial.polyval(2 * loc - 1, _legendre_monomials(m))
                  for m in range(k)]) * 2.0 ** (level / 2.0)  # (k, P), the same for every cell
    nodes = (np.arange(ncell)[:, None] + loc[None, :]) * h
    F = np.asarray(f(nodes.reshape(-1, 1)), np.float64).reshape(nodes.shape)
    return np.einsum("cp,mp,p->cm", F, B, wts).ravel()


class SparseGridOperator:
    """Device-backed derivative operators for one (D, k, n, scheme)."""

    def __init__(self, D, k, n, scheme="sparse", basis="hier"):
        """basis="pos" (D = 1 only) holds the position-basis operators of
        wave_evolve_1D; they run the plain form only."""
        self.D, self.k, self.n, self.scheme, self.basis = D, k, n, scheme, basis
        h = ctypes.c_void_p()
        if basis == "hier":
            check(lib().sgdg_op_create(D, k, n, _scheme(scheme), ctypes.byref(h)))
        elif basis == "pos":
            if D != 1:
                raise ValueError("the position basis is one-dimensional (D = 1)")
            check(lib().sgdg_op_create_1d(k, n, _lib.BASES["pos"], ctypes.byref(h)))
        else:
            raise ValueError("basis must be \"hier\" or \"pos\"")
        self._h = h
        self.N = get_size(D, k, n, scheme)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sgdg_op_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _len(self, which):
        return 2 * self.N if which == _lib.OP_WAVE_RHS else self.N

    def nnz(self, which):
        z = ctypes.c_int64()
        check(lib().sgdg_op_nnz(self._h, which, ctypes.byref(z)))
        return z.value

    def csr(self, which):
        """The assembled operator as scipy CSR (numerical zeros stored like the reference)."""
        m = self._len(which)
        return _csr_from(lambda p: lib().sgdg_op_nnz(self._h, which, p),
                         lambda a, b, c: lib().sgdg_op_export_csr(self._h, which, a, b, c), m)

    def device_csr(self, which):
        """The operator as the plain form holds it on the device, assembled on
        the GPU, copied back as scipy CSR (same entries as csr())."""
        m = self._len(which)
        return _csr_from(lambda p: lib().sgdg_op_device_nnz(self._h, which, p),
                         lambda a, b, c: lib().sgdg_op_export_device_csr(self._h, which, a, b, c), m)

    def apply(self, x, which=1, method="plain"):
        """y = A x on the GPU (host arrays in and out)."""
        x = np.ascontiguousarray(x, np.float64)
        if x.shape != (self._len(which),):
            raise ValueError("x must have %d entries" % self._len(which))
        y = np.empty_like(x)
        check(lib().sgdg_apply(self._h, which, _method(method), x, y))
        return y

    def apply_device(self, x_ptr, y_ptr, which=1, method="plain", stream=0):
        check(lib().sgdg_apply_device(self._h, which, _method(method), ctypes.c_void_p(x_ptr),
                                      ctypes.c_void_p(y_ptr), ctypes.c_void_p(stream)))

    def plain_steps_device(self, y_ptr, nsolves, dt, nsteps, which=-1, stream=0):
        """nsteps plain FP64 RK4 steps of y' = A y (A = operator `which`, the
        wave right-hand side by default) for nsolves device-resident states
        stored one after another at y_ptr, updated in place."""
        check(lib().sgdg_op_plain_steps_device(self._h, int(which), int(nsolves), ctypes.c_void_p(y_ptr), float(dt),
                                               int(nsteps), ctypes.c_void_p(stream)))


def D_matrix(D, d, k, n, scheme="sparse"):
    """D-dimensional derivative along dim d, 1-based (src/multidim_derivative.jl:61-65)."""
    return SparseGridOperator(D, k, n, scheme).csr(d)


def grad_matrix(D, k, n, scheme="sparse"):
    op = SparseGridOperator(D, k, n, scheme)
    return [op.csr(d) for d in range(1, D + 1)]


def laplacian_matrix(D, k, n, scheme="sparse"):
    return SparseGridOperator(D, k, n, scheme).csr(_lib.OP_LAPLACIAN)


# -------------------------------------------------------------- evolvers ----
def _steps(t0, t1, dt, nsteps):
    if nsteps is None:
        if dt is None:
            raise ValueError("give dt or nsteps (fixed-step classical RK4)")
        nsteps = int(round((t1 - t0) / dt))
        if nsteps < 1 or abs(nsteps * dt - (t1 - t0)) > 1e-9 * max(1.0, abs(t1 - t0)):
            raise ValueError("(t1 - t0) must be a whole number of steps dt")
    return int(nsteps)


def _order(order):
    if order != "rk4":
        # the reference accepts "45"/"78" (ODE.jl adaptive) and throws
        # ArgumentError(:order) otherwise (src/pdes.jl:62-68)
        raise ValueError("order: only fixed-step classical \"rk4\" is implemented on the GPU")


def wave_evolve(D, k, n, f0, v0, time0, time1, order="rk4", scheme="sparse", dt=None, nsteps=None, nout=2,
                method="plain", op=None):
    """u_tt = laplacian(u) on the periodic unit cube (src/pdes.jl:54-83).

    Returns (times, states): nout equally spaced states [f; v] of length 2N.
    f0, v0 are coefficient vectors or functions (projected with vcoeffs_DG)."""
    _order(order)
    if callable(f0):
        f0 = vcoeffs_DG(D, k, n, f0, scheme)
    if callable(v0):
        v0 = vcoeffs_DG(D, k, n, v0, scheme)
    op = op or SparseGridOperator(D, k, n, scheme)
    f0 = np.ascontiguousarray(f0, np.float64)
    v0 = np.ascontiguousarray(v0, np.float64)
    if f0.shape != (op.N,) or v0.shape != (op.N,):
        raise ValueError("f0 and v0 must have get_size(D,k,n) = %d entries" % op.N)
    ns = _steps(time0, time1, dt, nsteps)
    times = np.zeros(nout)
    states = np.zeros((nout, 2 * op.N))
    check(lib().sgdg_wave_evolve(op._h, f0, v0, float(time0), float(time1), ns, int(nout), _method(method), times,
                                 states.reshape(-1)))
    return times, list(states)


def advect_evolve(D, k, n, a, f0, time0, time1, order="rk4", scheme="sparse", dt=None, nsteps=None, nout=2,
                  method="plain", op=None):
    """f_t = -sum_d a_d D_d f on the periodic unit cube (operator composed
    from grad_matrix, src/multidim_derivative.jl:67-69).  Returns (times, states)."""
    _order(order)
    if callable(f0):
        f0 = vcoeffs_DG(D, k, n, f0, scheme)
    op = op or SparseGridOperator(D, k, n, scheme)
    a = np.ascontiguousarray(a, np.float64)
    f0 = np.ascontiguousarray(f0, np.float64)
    if a.shape != (D,):
        raise ValueError("a must have D entries")
    if f0.shape != (op.N,):
        raise ValueError("f0 must have get_size(D,k,n) = %d entries" % op.N)
    ns = _steps(time0, time1, dt, nsteps)
    times = np.zeros(nout)
    states = np.zeros((nout, op.N))
    check(lib().sgdg_advect_evolve(op._h, a, f0, float(time0), float(time1), ns, int(nout), _method(method), times,
                                   states.reshape(-1)))
    return times, list(states)


def norm_squared(coeffs, basis="hier"):
    """Sum of the squared coefficients (src/pdes.jl:228-235): the L2 norm
    squared in an orthonormal basis ("hier" or "pos")."""
    if basis not in ("hier", "pos"):
        raise NotImplementedError("nodal and point basis norms are not implemented (as in the reference)")
    c = np.asarray(coeffs, np.float64)
    return float(np.dot(c, c))


def wave_evolve_1D(k, max_level, f0, v0, time0, time1, basis="hier", order="rk4", dt=None, nsteps=None, nout=2,
                   method="plain"):
    """wave_evolve_1D (src/pdes.jl:89-121).  basis="hier": the 1D sparse grid
    is the full grid and the evolution is wave_evolve(1, ...).  basis="pos":
    functions are projected with pos_vcoeffs_DG, D_op is the position-basis
    periodic_DLF_matrix, the right-hand side is wave_data(D_op * D_op) and the
    plain FP64 form steps it on the GPU; states are [f; v] in the position
    basis.  The reference's "nodal" basis throws and its "point" basis is not
    built."""
    if basis == "pos":
        if method != "plain":
            raise ValueError("the position basis runs the plain form only")
        if callable(f0):
            f0 = pos_vcoeffs_DG(k, max_level, f0)
        if callable(v0):
            v0 = pos_vcoeffs_DG(k, max_level, v0)
        op = SparseGridOperator(1, k, max_level, basis="pos")
        return wave_evolve(1, k, max_level, f0, v0, time0, time1, order=order, dt=dt, nsteps=nsteps, nout=nout,
                           method=method, op=op)
    if basis != "hier":
        raise ValueError("basis must be \"hier\" or \"pos\" (nodal evolution throws in the reference; point is "
                         "not built)")
    return wave_evolve(1, k, max_level, f0, v0, time0, time1, order=order, dt=dt, nsteps=nsteps, nout=nout,
                       method=method)


def energy_func_1D(k, level, soln, basis="hier"):
    """||D u||^2 + ||u_t||^2 per stored state of a 1D solution
    (src/pdes.jl:237-255), D the periodic 1D operator of the basis ("hier"
    or "pos")."""
    if basis not in ("hier", "pos"):
        raise NotImplementedError("nodal and point basis norms are not implemented (as in the reference)")
    D_op = periodic_DLF_matrix(k, level, basis=basis)
    times, states = soln
    energies = []
    for st in states:
        st = np.asarray(st, np.float64)
        h = int(round(st.size / 2))
        energies.append(norm_squared(D_op @ st[:h]) + norm_squared(st[h:]))
    return np.array(times), np.array(energies)


def energy_func(D, k, n, soln, scheme="sparse", op=None):
    """sum_d ||D_d u||^2 + ||u_t||^2 per stored state (src/pdes.jl:258-273), D_d applied on the GPU."""
    op = op or SparseGridOperator(D, k, n, scheme)
    times, states = soln
    N = op.N
    energies = []
    for s in states:
        s = np.asarray(s, np.float64)
        u, ut = s[:N], s[N:]
        energies.append(sum(float(np.sum(op.apply(u, d) ** 2)) for d in range(1, D + 1)) + float(np.sum(ut ** 2)))
    return np.array(times), np.array(energies)


# ------------------------------------------------- nodal bases, Vlasov ----
_TRANSFORMS = {("modal", "nodal"): 0, ("nodal", "points"): 1, ("points", "nodal"): 2, ("nodal", "modal"): 3}


def _transform_id(frm, to):
    if (frm, to) not in _TRANSFORMS:
        raise ValueError("transforms: modal->nodal, nodal->points, points->nodal, nodal->modal")
    return _TRANSFORMS[(frm, to)]


def transform_1D(k, n, frm, to):
    """transform_1D(k, n, from, to) (src/1d_nodal_basis.jl:350-414), CSR."""
    w = _transform_id(frm, to)
    L = lib()
    return _csr_from(lambda p: L.sgdg_transform_1d_nnz(k, n, w, p),
                     lambda a, b, c: L.sgdg_transform_1d_export(k, n, w, a, b, c), k << n)


def transform(D, k, n, frm, to, scheme="sparse", device=False):
    """transform(D, k, n, from, to) (src/multidim_nodal_basis.jl:83-124), CSR;
    ``device=True`` assembles it on the GPU (the same entries and values)."""
    w = _transform_id(frm, to)
    sc = _scheme(scheme)
    L = lib()
    if device:
        nnz = ctypes.c_int64()
        check(L.sgdg_transform_device_export(D, k, n, sc, w, ctypes.byref(nnz), None, None, None))
        N = get_size(D, k, n, scheme)
        rp = np.empty(N + 1, np.int64)
        cl = np.empty(nnz.value, np.int32)
        vl = np.empty(nnz.value, np.float64)
        check(L.sgdg_transform_device_export(D, k, n, sc, w, ctypes.byref(nnz), rp.ctypes.data_as(ctypes.c_void_p),
                                             cl.ctypes.data_as(ctypes.c_void_p), vl.ctypes.data_as(ctypes.c_void_p)))
        return sp.csr_matrix((vl, cl, rp), shape=(N, N))
    return _csr_from(lambda p: L.sgdg_transform_nnz(D, k, n, sc, w, p),
                     lambda a, b, c: L.sgdg_transform_export(D, k, n, sc, w, a, b, c), get_size(D, k, n, scheme))


def make_modal2point_matrices(D, k, n):
    """(m2n, n2p), src/multidim_nodal_basis.jl:127-133 (D = phase-space dimensions)."""
    return transform(D, k, n, "modal", "nodal"), transform(D, k, n, "nodal", "points")


def make_point2modal_matrices(D, k, n):
    """(p2n, n2m), src/multidim_nodal_basis.jl:135-141."""
    return transform(D, k, n, "points", "nodal"), transform(D, k, n, "nodal", "modal")


def get_one_modal(D, k, n, scheme="sparse"):
    """Coefficients of f = 1 (src/basic_function_exact_coeffs.jl:5-8)."""
    out = np.zeros(get_size(D, k, n, scheme))
    out[0] = 1.0
    return out


def get_xi_modal(D, i, k, n, scheme="sparse"):
    """Coefficients of f = 2 x_i - 1 (src/basic_function_exact_coeffs.jl:11-17), i 1-based."""
    one = np.zeros(k << n)
    one[0] = 1.0
    xi = np.zeros(k << n)
    xi[1] = 1.0 / np.sqrt(3.0)
    return tensor_construct(D, k, n, [xi if d == i else one for d in range(1, D + 1)], scheme)


def get_xi_point(D, i, k, n, m2n, n2p):
    """Point values of 2 x_i - 1 (src/basic_function_exact_coeffs.jl:39-43)."""
    return n2p @ (m2n @ get_xi_modal(D, i, k, n))


class VlasovOperator:
    """Operators of vlasov_evolve for D space dimensions (phase space x_1..x_D,
    p_1..p_D on [0,1]^(2D), velocity 2 p_d - 1), k in {2, 3, 5}."""

    def __init__(self, D, k, n, scheme="sparse"):
        h = ctypes.c_void_p()
        check(lib().sgdg_vlasov_create(D, k, n, _scheme(scheme), ctypes.byref(h)))
        self._h = h
        self.D, self.k, self.n = D, k, n
        z = ctypes.c_int64()
        check(lib().sgdg_vlasov_size(self._h, ctypes.byref(z)))
        self.N = z.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sgdg_vlasov_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def v_point(self):
        out = np.zeros(self.D * self.N)
        check(lib().sgdg_vlasov_v_point(self._h, out))
        return out.reshape(self.D, self.N)

    def transform(self, frm, to):
        w = _transform_id(frm, to)
        L = lib()
        return _csr_from(lambda p: L.sgdg_vlasov_transform_nnz(self._h, w, p),
                         lambda a, b, c: L.sgdg_vlasov_transform_export(self._h, w, a, b, c), self.N)

    def _force(self, F_point):
        F = np.ascontiguousarray(np.asarray(F_point, np.float64).reshape(self.D, self.N)).reshape(-1)
        return F

    def rhs(self, F_point, f):
        out = np.zeros(self.N)
        check(lib().sgdg_vlasov_rhs(self._h, self._force(F_point), np.ascontiguousarray(f, np.float64), out))
        return out

    def write_h5(self, path="vlasov.h5", times=None, states=None):
        """The file vlasov_evolve writes (src/pdes.jl:145-163, 217-223):
        dimensions, order, levels; m2n, n2p, p2n, n2m and Ds[1] .. Ds[2D] as
        SparseMatrixCSC fields (.m, .n, .colptr, .rowval 1-based, .nzval);
        with a solution also times and f_modal.%06d.  HDF5, written on the
        host."""
        if times is None:
            check(lib().sgdg_vlasov_write_h5(self._h, os.fsencode(path), 0, None, None))
            return
        t = np.ascontiguousarray(times, np.float64).reshape(-1)
        S = np.ascontiguousarray(np.asarray(states, np.float64).reshape(t.size, self.N))
        check(lib().sgdg_vlasov_write_h5(self._h, os.fsencode(path), t.size, t.ctypes.data, S.ctypes.data))


def vlasov_evolve(D, k, n, F_point, f0_modal, time0, time1, nout=2, order="rk4", scheme="sparse", dt=None,
                  nsteps=None, op=None, method="plain", h5=None):
    """vlasov_evolve (src/pdes.jl:131-227) with classical RK4 and fixed steps:
    df/dt = -(v . grad_x f) + F . grad_p f, products taken in the point basis.
    ``F_point`` holds D arrays of point values.  method "plain": assembled
    FP64 sparse operators; "matfree": FP32 pencil sweeps, FP64 RK state.
    ``h5``: a path (the reference always writes "vlasov.h5") to receive the
    operators and the stored states as the reference writes them.
    Returns (times, states)."""
    _order(order)
    op = op or VlasovOperator(D, k, n, scheme)
    f0 = np.ascontiguousarray(f0_modal, np.float64)
    if f0.shape != (op.N,):
        raise ValueError("f0 must have %d entries" % op.N)
    ns = _steps(time0, time1, dt, nsteps)
    times = np.zeros(nout)
    states = np.zeros((nout, op.N))
    check(lib().sgdg_vlasov_evolve(op._h, op._force(F_point), f0, float(time0), float(time1), ns, int(nout),
                                   _method(method), times, states.reshape(-1)))
    if h5 is not None:
        op.write_h5(h5, times, states)
    return times, list(states)


# ------------------------------------------------------------ evaluation ----
def reconstruct_DG(D, k, n, coeffs, xs, scheme="sparse"):
    """Value of the expansion with coefficient vector ``coeffs`` (the
    reference's vector layout) at ``xs``: reconstruct_DG
    (src/dg_methods.jl:150-165), batched and in FP64 on the GPU.  ``xs`` of
    D coordinates gives a float; an (npts, D) array gives npts values.  A
    coordinate below 0 or NaN raises SGDGError (code SGDG_EINVAL)."""
    c = np.ascontiguousarray(coeffs, np.float64)
    N = get_size(D, k, n, scheme)
    if c.shape != (N,):
        raise ValueError("coeffs must have %d entries" % N)
    x = np.asarray(xs, np.float64)
    single = x.ndim == 1
    if x.shape[-1] != D or x.ndim > 2:
        raise ValueError("xs must have D = %d coordinates per point" % D)
    x = np.ascontiguousarray(x.reshape(-1, D))
    out = np.empty(x.shape[0])
    check(lib().sgdg_evaluate(D, k, n, _scheme(scheme), c, x.shape[0], x.reshape(-1), out))
    return float(out[0]) if single else out


class DGFunction:
    """A coefficient vector as a function of points, evaluated on the GPU:
    ``f(x)`` for x of D coordinates, or an (npts, D) array of points."""

    def __init__(self, D, k, n, coeffs, scheme="sparse"):
        self.D, self.k, self.n, self.scheme = D, k, n, scheme
        self.coeffs = np.ascontiguousarray(coeffs, np.float64)

    def __call__(self, xs):
        return reconstruct_DG(self.D, self.k, self.n, self.coeffs, xs, self.scheme)


def _values(f, pts):
    """f at every row of pts: one vectorised call when f takes an (npts, D)
    array (a DGFunction or a numpy expression), else one call per point
    with the point as a tuple, as the reference's functions take it."""
    try:
        v = np.asarray(f(pts), np.float64)
        if v.shape == (pts.shape[0],):
            return v
    except Exception:
        pass
    return np.array([float(f(tuple(p))) for p in pts])


def monte_carlo(f, D, count=1000, rng=None):
    """Mean of f over ``count`` uniform points of [0, 1]^D (src/error_measure.jl:12-19)."""
    rng = rng if rng is not None else np.random.default_rng()
    return float(np.mean(_values(f, rng.random((count, D)))))


def mcerr(f, g, D, count=1000, rng=None):
    """Root-mean-square of f - g over ``count`` uniform points of [0, 1]^D
    (src/error_measure.jl:39-41); f or g may be a DGFunction (GPU)."""
    rng = rng if rng is not None else np.random.default_rng()
    pts = rng.random((count, D))
    return float(np.sqrt(np.mean((_values(f, pts) - _values(g, pts)) ** 2)))


def mcerr2(f, g, D, batch=50, Z=1.0, rng=None):
    """mcerr with the adaptive batching of monte_carlo2
    (src/error_measure.jl:21-37, 43-45): batches of ``batch`` points until a
    new batch's mean is within Z standard deviations of the earlier batch
    means."""
    rng = rng if rng is not None else np.random.default_rng()
    means = []
    while True:
        pts = rng.random((batch, D))
        sq = (_values(f, pts) - _values(g, pts)) ** 2
        if len(means) > 1 and abs(np.mean(sq) - np.mean(means)) / np.std(means, ddof=1) < Z:
            break
        means.append(float(np.mean(sq)))
    return float(np.sqrt(np.mean(means)))


# --------------------------------------------------------------- batches ----
class Batch:
    """Independent solves of uneven (D, k, n) advanced together by the
    matrix-free FP32/FP64 engine (one persistent launch per RK4 step,
    replayed from a CUDA graph)."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().sgdg_batch_create(ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sgdg_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, kind, D, k, n, y0, dt, a=None, scheme="sparse"):
        kinds = {"advect": _lib.KIND_ADVECT, "wave": _lib.KIND_WAVE}
        if kind not in kinds:
            raise ValueError("kind must be \"advect\" or \"wave\"")
        y0 = np.ascontiguousarray(y0, np.float64)
        ap = None
        if a is not None:
            a_arr = np.ascontiguousarray(a, np.float64)
            ap = a_arr.ctypes.data_as(ctypes.c_void_p)
        i = ctypes.c_int()
        check(lib().sgdg_batch_add(self._h, kinds[kind], D, k, n, _scheme(scheme), ap, float(dt), y0,
                                   ctypes.byref(i)))
        return i.value

    def add_vlasov(self, Dx, k, n, f0, F_point, dt, scheme="sparse"):
        """A Vlasov solve (phase space of 2 Dx dimensions, k in {2, 3, 5})."""
        f0 = np.ascontiguousarray(f0, np.float64)
        F = np.ascontiguousarray(np.asarray(F_point, np.float64).reshape(Dx, f0.size)).reshape(-1)
        i = ctypes.c_int()
        check(lib().sgdg_batch_add_vlasov(self._h, Dx, k, n, _scheme(scheme), float(dt), F, f0, ctypes.byref(i)))
        return i.value

    def remove(self, sid):
        check(lib().sgdg_batch_remove(self._h, sid))

    def set_stream(self, stream):
        check(lib().sgdg_batch_set_stream(self._h, ctypes.c_void_p(stream)))

    def step(self, nsteps=1):
        check(lib().sgdg_batch_step(self._h, int(nsteps)))

    def state_size(self, sid):
        z = ctypes.c_int64()
        check(lib().sgdg_batch_state_size(self._h, sid, ctypes.byref(z)))
        return z.value

    def state(self, sid):
        y = np.empty(self.state_size(sid))
        check(lib().sgdg_batch_get_state(self._h, sid, y))
        return y

    def total_size(self):
        z = ctypes.c_int64()
        check(lib().sgdg_batch_total_size(self._h, ctypes.byref(z)))
        return z.value

    def upload(self, ptr):
        """All live states from host memory at address ``ptr`` (float64, id order)."""
        check(lib().sgdg_batch_upload(self._h, ctypes.c_void_p(ptr)))

    def download(self, ptr):
        """All live states into host memory at address ``ptr`` (synchronises)."""
        check(lib().sgdg_batch_download(self._h, ctypes.c_void_p(ptr)))

    def step_host(self, y_in, y_out=None, nsteps=1, chunks=16):
        """Every live state from host memory, ``nsteps`` RK4 steps, the results
        back (id order, like upload/download).  ``y_in`` / ``y_out`` are
        addresses of float64 host memory (pinned for the copies to overlap the
        steps) or numpy arrays; ``y_out`` defaults to ``y_in``."""
        keep = []

        def addr(a):
            if isinstance(a, np.ndarray):
                if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size != self.total_size():
                    raise ValueError("need a C-contiguous float64 array of total_size() entries")
                keep.append(a)
                return a.ctypes.data
            return int(a)
        pin = addr(y_in)
        pout = pin if y_out is None else addr(y_out)
        check(lib().sgdg_batch_step_host(self._h, ctypes.c_void_p(pin), ctypes.c_void_p(pout), int(nsteps),
                                         int(chunks)))

    def autotune(self):
        """Tunes the tile shape of every (D, k) in the batch not tuned yet;
        returns how many were tuned."""
        n = ctypes.c_int()
        check(lib().sgdg_batch_autotune(self._h, ctypes.byref(n)))
        return n.value

    def step_info(self):
        launches = ctypes.c_int64()
        dofs = ctypes.c_double()
        check(lib().sgdg_batch_step_info(self._h, ctypes.byref(launches), ctypes.byref(dofs)))
        return launches.value, dofs.value


# -------------------------------------------------------------- serving ----
class Server:
    """Request loop over the matrix-free engine (continuous batching): queued
    solves are admitted in arrival order while the HBM budget has room, run
    together in shared launches, and leave when their steps are done.  Times
    are seconds on the server's steady clock (``clock()``)."""

    QUEUED, RUNNING, DONE, FAILED, CANCELLED = range(5)

    def __init__(self, max_chunk_steps=25):
        h = ctypes.c_void_p()
        check(lib().sgdg_server_create(int(max_chunk_steps), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sgdg_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        check(lib().sgdg_server_set_stream(self._h, ctypes.c_void_p(stream)))

    def clock(self):
        t = ctypes.c_double()
        check(lib().sgdg_server_clock(self._h, ctypes.byref(t)))
        return t.value

    def submit(self, kind, D, k, n, y0, dt, nsteps, a=None, scheme="sparse", t_arrival=-1.0):
        kinds = {"advect": _lib.KIND_ADVECT, "wave": _lib.KIND_WAVE}
        if kind not in kinds:
            raise ValueError("kind must be \"advect\" or \"wave\"")
        y0 = np.ascontiguousarray(y0, np.float64)
        ap = None
        if a is not None:
            a_arr = np.ascontiguousarray(a, np.float64)
            ap = a_arr.ctypes.data_as(ctypes.c_void_p)
        rid = ctypes.c_int64()
        check(lib().sgdg_server_submit(self._h, kinds[kind], D, k, n, _scheme(scheme), ap, float(dt), y0,
                                       int(nsteps), float(t_arrival), ctypes.byref(rid)))
        return rid.value

    def tick(self):
        """One admit / advance / retire round; returns the number finished."""
        c = ctypes.c_int()
        check(lib().sgdg_server_tick(self._h, ctypes.byref(c)))
        return c.value

    def status(self, rid):
        """(state, steps_done, t_arrival, t_admit, t_done)."""
        st, sd = ctypes.c_int(), ctypes.c_int64()
        ta, tb, tc = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().sgdg_server_status(self._h, int(rid), ctypes.byref(st), ctypes.byref(sd), ctypes.byref(ta),
                                       ctypes.byref(tb), ctypes.byref(tc)))
        return st.value, sd.value, ta.value, tb.value, tc.value

    def result(self, rid, size):
        y = np.empty(int(size))
        check(lib().sgdg_server_result(self._h, int(rid), y))
        return y

    def snapshot(self, rid, size):
        """Checkpoint of a request: (state now, steps done).  Submitting the
        state for the remaining steps resumes the solve bit for bit."""
        y = np.empty(int(size))
        done = ctypes.c_int64()
        check(lib().sgdg_server_snapshot(self._h, int(rid), y, ctypes.byref(done)))
        return y, done.value

    def cancel(self, rid):
        check(lib().sgdg_server_cancel(self._h, int(rid)))

    def counts(self):
        """(queued, running, finished not yet collected, DOF-updates so far)."""
        q, r, f = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        d = ctypes.c_double()
        check(lib().sgdg_server_counts(self._h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(f), ctypes.byref(d)))
        return q.value, r.value, f.value, d.value


def tile_shape(D, k):
    """(wlog, coop, tuned) of the pencil tiles of (D, k): 2^wlog scales the
    tile width, row levels <= lmax - coop are swept by whole warps."""
    w, c, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(lib().sgdg_tile_shape(D, k, ctypes.byref(w), ctypes.byref(c), ctypes.byref(t)))
    return w.value, c.value, bool(t.value)


def set_tile_shape(D, k, wlog, coop):
    check(lib().sgdg_set_tile_shape(D, k, wlog, coop))


def clear_tile_shapes():
    check(lib().sgdg_clear_tile_shapes())


def set_hbm_budget(nbytes):
    check(lib().sgdg_set_hbm_budget(int(nbytes)))


def hbm_in_use():
    z = ctypes.c_int64()
    check(lib().sgdg_hbm_in_use(ctypes.byref(z)))
    return z.value


def sync():
    check(lib().sgdg_sync())
