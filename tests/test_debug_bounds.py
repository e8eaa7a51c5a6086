"""The debug build's device index checks (SGDG_DEBUG=1): every gather and
scatter index of the matrix-free stage kernel, the CSR kernels and the device
assembly is checked against the length of the vector it addresses, a failed
check is counted and its access skipped (no trap, no fault).  The GPU test
runs parity shapes of every kernel family on that build, in a fresh process
that loads the debug library, and requires zero failed checks and results
that still match the FP64 oracle."""
import ctypes
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import ctypes, importlib, sys
import numpy as np
sys.path.insert(0, ROOT)
import __graft_entry__ as g
sg = g.load_package(build=True)
from oracle import oracle as O
L = sg._lib.lib()
assert L._name.endswith("_build_debug/libsgdg.so"), L._name
checked, viol = ctypes.c_int(), ctypes.c_int64()
sg.check(L.sgdg_debug_bounds(ctypes.byref(checked), ctypes.byref(viol), 1))
assert checked.value == 1
rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
rng = np.random.default_rng(3)
# plain CSR and matrix-free applications, several (D, k, n)
for D, k, n in [(2, 3, 4), (3, 2, 3), (2, 5, 3), (1, 4, 5), (2, 3, 10)]:
    op = sg.SparseGridOperator(D, k, n)
    x = rng.standard_normal(op.N)
    for d in range(1, D + 1):
        ref = O.spmv_csc(O.D_matrix_raw(D, d, k, n), x)
        assert rel(op.apply(x, d, "plain"), ref) < 1e-10
        assert rel(op.apply(x, d, "matfree"), ref) < 5e-7
    assert rel(op.apply(x, 0, "matfree"), O.spmv_csc(O.laplacian_matrix_raw(D, k, n), x)) < 1e-6
    op.device_csr(-1)
    op.close()
# a mixed batch: wave (squared and doubled sweeps), advection, Vlasov
serving = importlib.import_module(sg.__name__ + ".serving")
W = importlib.import_module(sg.__name__ + ".workloads")
b = sg.Batch()
for kind, D, k, n in [("wave", 3, 3, 5), ("advect", 2, 4, 5), ("advect", 3, 2, 4), ("wave", 2, 2, 6)]:
    N = sg.get_size(D, k, n)
    y0 = rng.standard_normal(2 * N if kind == "wave" else N) * 1e-2
    b.add(kind, D, k, n, y0, 1e-3, a=rng.uniform(-1, 1, D) if kind == "advect" else None)
F, f0 = W.vlasov_case(sg, 1, 2, 4, seed=5)
b.add_vlasov(1, 2, 4, f0, F, 1e-3)
b.autotune()
b.step(5)
b.close()
# device transforms, warp rows and block rows
for D, k, n in [(2, 3, 4), (6, 2, 3)]:
    sg.transform(D, k, n, "modal", "nodal", device=True)
sg.vlasov_evolve(1, 2, 4, F, f0, 0.0, 5e-3, nsteps=5, method="plain")
sg.check(L.sgdg_debug_bounds(ctypes.byref(checked), ctypes.byref(viol), 0))
print("bounds checks failed:", viol.value)
assert viol.value == 0
'''


def test_release_build_reports_no_checks(sgdg):
    checked, viol = ctypes.c_int(7), ctypes.c_int64(7)
    assert sgdg.lib().sgdg_debug_bounds(ctypes.byref(checked), ctypes.byref(viol), 0) == 0
    assert checked.value == 0 and viol.value == 0


@pytest.mark.gpu
def test_debug_build_runs_parity_shapes_without_a_failed_check():
    env = dict(os.environ, SGDG_DEBUG="1")
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + SCRIPT], env=env, capture_output=True,
                       text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "bounds checks failed: 0" in r.stdout
