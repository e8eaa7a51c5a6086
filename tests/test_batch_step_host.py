"""Batch.step_host: host states in, RK4 steps, host states out, with the
batch's groups split into pipeline chunks on their own streams.  Each chunk
runs the same tiles as the whole batch, so the states must equal (bitwise)
upload + step + download, for any chunk count, from pageable or pinned
buffers, and with solves of several classes added in interleaved order."""
import numpy as np
import pytest


def mixed_batch(sgdg):
    rng = np.random.default_rng(12)
    b = sgdg.Batch()
    specs = []
    for i in range(14):
        if i % 3 == 0:
            N = sgdg.get_size(3, 3, 4)
            y0 = np.concatenate([sgdg.fourier_coeffs(3, 3, 4, [((1, 2, 1), 0.5, "sin", 0.0)]), np.zeros(N)])
            b.add("wave", 3, 3, 4, y0, 2e-3)
        else:
            y0 = rng.standard_normal(sgdg.get_size(2, 2, 5)) * 0.1
            b.add("advect", 2, 2, 5, y0, 1e-3, a=[0.6, -0.2 * i])
        specs.append(y0)
    return b, np.concatenate(specs)


@pytest.mark.gpu
@pytest.mark.parametrize("chunks", [1, 2, 3, 8])
def test_step_host_equals_upload_step_download(sgdg, chunks):
    b, y = mixed_batch(sgdg)
    ref = y.copy()
    b.upload(ref.ctypes.data)
    b.step(3)
    b.download(ref.ctypes.data)
    b2, y2 = mixed_batch(sgdg)
    out = np.empty_like(y2)
    b2.step_host(y2, out, nsteps=3, chunks=chunks)
    assert np.array_equal(out, ref)
    # in place, twice: the same as six steps
    b2.step_host(y2, nsteps=3, chunks=chunks)
    b2.step_host(y2, nsteps=3, chunks=chunks)
    b.step(3)
    b.download(ref.ctypes.data)
    assert np.array_equal(y2, ref)
    b.close()
    b2.close()


@pytest.mark.gpu
def test_step_host_on_an_empty_batch(sgdg):
    b = sgdg.Batch()
    y = np.zeros(0)
    b.step_host(y.ctypes.data, y.ctypes.data, nsteps=2, chunks=4)  # nothing to move or step
    b.close()


@pytest.mark.gpu
def test_step_host_rejects_a_wrong_size(sgdg):
    b = sgdg.Batch()
    with pytest.raises(ValueError):
        b.step_host(np.zeros(3), nsteps=1)
    b.close()


def _pinned(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory()


@pytest.mark.gpu
def test_single_step_between_pinned_buffers(sgdg):
    """One step between pinned buffers (the copies asynchronous, overlapping
    the other chunks' steps): the same bits as upload + step + download, call
    after call, in place too, and after the batch changes (chunk lists
    rebuilt)."""
    torch = pytest.importorskip("torch")
    b, y = mixed_batch(sgdg)
    ref1 = y.copy()
    b.upload(ref1.ctypes.data)
    b.step(1)
    b.download(ref1.ctypes.data)
    b.step(1)
    ref2 = np.empty_like(y)
    b.download(ref2.ctypes.data)
    b2, y2 = mixed_batch(sgdg)
    hin, hout = _pinned(torch, y2), _pinned(torch, np.zeros_like(y2))
    for _ in range(3):  # a new epoch each call
        b2.step_host(hin.data_ptr(), hout.data_ptr(), 1)
        assert np.array_equal(hout.numpy(), ref1)
    b2.step_host(hin.data_ptr(), None, 1)
    b2.step_host(hin.data_ptr(), None, 1)
    assert np.array_equal(hin.numpy(), ref2)
    # a solve joins: the host-to-host list is rebuilt
    extra = np.random.default_rng(5).standard_normal(sgdg.get_size(2, 2, 5)) * 0.1
    b.add("advect", 2, 2, 5, extra, 1e-3, a=[0.3, 0.4])
    b2.add("advect", 2, 2, 5, extra, 1e-3, a=[0.3, 0.4])
    y3 = np.concatenate([ref2, extra])
    ref3 = y3.copy()
    b.upload(ref3.ctypes.data)
    b.step(1)
    b.download(ref3.ctypes.data)
    h3 = _pinned(torch, y3)
    b2.step_host(h3.data_ptr(), None, 1)
    assert np.array_equal(h3.numpy(), ref3)
    b.close()
    b2.close()


@pytest.mark.gpu
def test_single_step_between_pinned_buffers_several_groups(sgdg):
    """A class large enough for several groups, so the chunks hold different
    groups."""
    torch = pytest.importorskip("torch")
    def batch():
        b = sgdg.Batch()
        ys = []
        for i in range(100):
            f0 = sgdg.fourier_coeffs(3, 3, 6, [((1 + i % 3, 2, 1), 0.5, "sin", 0.1 * i)])
            y0 = np.concatenate([f0, np.zeros_like(f0)])
            b.add("wave", 3, 3, 6, y0, 2e-3)
            ys.append(y0)
        return b, np.concatenate(ys)
    b, y = batch()
    ref = y.copy()
    b.upload(ref.ctypes.data)
    b.step(1)
    b.download(ref.ctypes.data)
    b2, y2 = batch()
    h = _pinned(torch, y2)
    b2.step_host(h.data_ptr(), None, 1)
    assert np.array_equal(h.numpy(), ref)
    b.close()
    b2.close()
