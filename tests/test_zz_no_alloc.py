"""sgdg_apply_noalloc: the matrix-free operator application for callers that
cannot allocate device memory (their device memory belongs to another
allocator, their runtime forbids allocation after start-up, or they cannot
take cudaMalloc's device-wide synchronisation).  Its scratch is a fixed
16 MiB device array inside the library, so the call allocates nothing.

The test calls it through the C ABI twice in a row (different operators and
inputs) and compares each result with the existing device entry point
(sgdg_apply_device, matrix-free method), within the matrix-free apply
tolerance used by the other parity tests.  This file is collected last so a
run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 5e-7  # relative L2, as for the matrix-free applications in test_gpu_parity.py


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _existing(sgdg, torch, op, which, x):
    y = torch.empty_like(x)
    sgdg.check(sgdg.lib().sgdg_apply_device(op._h, which, 1, ctypes.c_void_p(x.data_ptr()),
                                            ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(0)))
    torch.cuda.synchronize()
    return y.cpu().numpy()


def _noalloc(sgdg, torch, D, k, n, which, x):
    y = torch.empty_like(x)
    code = sgdg.lib().sgdg_apply_noalloc(D, k, n, 0, which, ctypes.c_void_p(x.data_ptr()),
                                         ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(0))
    sgdg.check(code)
    return y.cpu().numpy()


def test_noalloc_matches_existing_entry_point_twice(sgdg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    D, k, n = 3, 3, 5
    op = sgdg.SparseGridOperator(D, k, n)
    rng = np.random.default_rng(42)
    in_use = sgdg.hbm_in_use()
    calls = [(2, rng.standard_normal(op.N)), (0, rng.standard_normal(op.N))]  # D_2, then the Laplacian
    free_after = []
    for which, xh in calls:
        x = torch.tensor(xh, dtype=torch.float64, device="cuda")
        ref = _existing(sgdg, torch, op, which, x)
        torch.cuda.synchronize()
        got = _noalloc(sgdg, torch, D, k, n, which, x)
        free_after.append(torch.cuda.mem_get_info()[0])
        assert _rel(got, ref) <= TOL, (which, _rel(got, ref))
    # the library's own device allocations are untouched by the no-alloc calls
    assert sgdg.hbm_in_use() >= in_use
    # a third call on the same device frees and takes no device memory
    x = torch.tensor(calls[0][1], dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    sgdg.check(sgdg.lib().sgdg_apply_noalloc(D, k, n, 0, 2, ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(0)))
    assert torch.cuda.mem_get_info()[0] == before


# Shapes that take every path of the entry point: k <= 3 (four columns per
# thread) and k = 4, 5 (two), D = 1 (one phase, no wait), the 1D table in
# shared memory and (k = 3, n = 10: ~82 KB) in global memory.
SHAPES = [(1, 2, 6), (2, 5, 5), (4, 4, 4), (1, 3, 10), (3, 2, 4)]


@pytest.mark.parametrize("D,k,n", SHAPES)
def test_noalloc_shapes_match_existing_and_oracle(sgdg, O, D, k, n):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    op = sgdg.SparseGridOperator(D, k, n)
    rng = np.random.default_rng(7 + D + 10 * k + 100 * n)
    for which in list(range(1, D + 1)) + [0]:
        xh = rng.standard_normal(op.N)
        x = torch.tensor(xh, dtype=torch.float64, device="cuda")
        ref = _existing(sgdg, torch, op, which, x)
        got = _noalloc(sgdg, torch, D, k, n, which, x)
        assert _rel(got, ref) <= TOL, (which, _rel(got, ref))
        # and against the FP64 oracle's assembled operator
        A = O.laplacian_matrix_raw(D, k, n) if which == 0 else O.D_matrix_raw(D, which, k, n)
        assert _rel(got, O.spmv_csc(A, xh)) <= TOL, (which, "oracle")
    op.close()


def test_noalloc_leaves_planned_engines_launchable(sgdg):
    # The kernel's dynamic shared-memory limit is process-wide: a no-alloc
    # call on a small problem must not lower it below what an engine planned
    # for a larger one, or that engine's next launch would be refused.
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    big = sgdg.SparseGridOperator(3, 3, 6)
    rng = np.random.default_rng(3)
    xb = torch.tensor(rng.standard_normal(big.N), dtype=torch.float64, device="cuda")
    first = _existing(sgdg, torch, big, 1, xb)
    xs = torch.tensor(rng.standard_normal(sgdg.get_size(2, 2, 3)), dtype=torch.float64, device="cuda")
    _noalloc(sgdg, torch, 2, 2, 3, 1, xs)
    again = _existing(sgdg, torch, big, 1, xb)
    assert np.array_equal(first, again)
    big.close()


def test_noalloc_rejects_problems_beyond_its_scratch(sgdg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    D, k, n = 5, 3, 8  # 5.68M coefficients: FP32 staging and partial sums alone take 43 MiB
    N = sgdg.get_size(D, k, n)
    x = torch.zeros(N, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    code = sgdg.lib().sgdg_apply_noalloc(D, k, n, 0, 1, ctypes.c_void_p(x.data_ptr()),
                                         ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(0))
    assert code == 1
    assert "at most" in sgdg._lib.last_error()
