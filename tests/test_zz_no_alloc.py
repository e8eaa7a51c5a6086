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
