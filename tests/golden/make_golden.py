"""Writes the golden fixtures of tests/test_golden.py from the FP64 oracle.

The reference (Julia) cannot run in this environment, so these vectors are
the oracle's outputs on small seeded cases, frozen: they pin the oracle and
the product against silent drift.  The oracle itself is pinned against the
reference's own known-answer tests (tests/test_oracle_*.py).

    python tests/golden/make_golden.py     # rewrites tests/golden/*.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def modes(D, seed, count=3):
    rng = np.random.default_rng(seed)
    return [(tuple(int(v) for v in rng.integers(1, 4, D)), float(rng.uniform(-1, 1)),
             "sin" if rng.random() < 0.5 else "cos", 0.0) for _ in range(count)]


def csr_dict(prefix, A):
    A = A.tocsr()
    A.sort_indices()
    return {prefix + "_indptr": A.indptr.astype(np.int64), prefix + "_indices": A.indices.astype(np.int32),
            prefix + "_data": A.data}


def main():
    out = {}
    # index map and 1D operator
    L, C, M = O.index_map(3, 2, 3)
    out.update(index_L=L, index_C=C, index_M=M)
    out.update(csr_dict("dlf_k3_n3", O.periodic_DLF_matrix(3, 3)))
    # D_2 and the Laplacian, D=2 k=2 n=3
    out.update(csr_dict("d2_D2k2n3", O.D_matrix(2, 2, 2, 3)))
    out.update(csr_dict("lap_D2k2n3", O.laplacian_matrix(2, 2, 3)))
    # 40 RK4 steps of the 2D wave, k=3 n=3
    D, k, n = 2, 3, 3
    f0 = O.fourier_coeffs(D, k, n, modes(D, 1))
    v0 = O.fourier_coeffs(D, k, n, modes(D, 2))
    y0 = np.concatenate([f0, v0])
    out.update(wave_y0=y0, wave_y40=O.CSR(O.wave_rhs_raw(D, k, n)).rk4(y0, 2e-3, 40, nthreads=1))
    # 40 RK4 steps of 3D advection, k=2 n=3
    a = np.array([0.7, -0.3, 0.2])
    g0 = O.fourier_coeffs(3, 2, 3, modes(3, 3))
    out.update(adv_a=a, adv_y0=g0, adv_y40=O.CSR(O.advection_matrix_raw(3, 2, 3, a)).rk4(g0, 2e-3, 40, nthreads=1))
    # nodal transforms, k=2 n=3 (1D) and D=2 k=3 n=2
    out.update(csr_dict("m2n_1d_k2n3", O.transform_1D(2, 3, "modal", "nodal")))
    out.update(csr_dict("n2p_D2k3n2", O.transform(2, 3, 2, "nodal", "points")))
    # Vlasov right-hand side, D=1 (phase space 2D), k=2 n=3
    ops = O.vlasov_operators(1, 2, 3)
    N = O.get_size(2, 2, 3)
    rng = np.random.default_rng(4)
    F = rng.uniform(-0.1, 0.1, (1, N))
    f = O.fourier_coeffs(2, 2, 3, modes(2, 5))
    out.update(vlasov_F=F, vlasov_f=f, vlasov_rhs=O.vlasov_rhs(1, 2, 3, ops, F, f))
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **out)
    print("wrote", os.path.join(HERE, "oracle_small.npz"), sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    main()
