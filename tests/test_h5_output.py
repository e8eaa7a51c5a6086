"""The reference's vlasov.h5 output (src/pdes.jl:145-163 operators,
:217-223 solution) written by sgdg_vlasov_write_h5: every dataset name, the
operators as SparseMatrixCSC fields (1-based colptr and rowval, the product's
operators bit for bit and the oracle's to roundoff), times and the states,
read back with a reader that checks the HDF5 structures field by field
(tests/h5spec.py).  No HDF5 library is available to read the file
independently; the structures follow the published file format
specification."""
import os

import numpy as np
import pytest

from h5spec import read

WHICH = {"m2n": ("modal", "nodal"), "n2p": ("nodal", "points"), "p2n": ("points", "nodal"),
         "n2m": ("nodal", "modal")}


def csc_fields(A):
    C = A.tocsc()
    C.sort_indices()
    return C.shape[0], C.shape[1], C.indptr.astype(np.int64) + 1, C.indices.astype(np.int64) + 1, C.data


def check_operator(f, name, A, exact=True, ref=None):
    m, n, colptr, rowval, nzval = csc_fields(A)
    assert f[name + ".m"] == m and f[name + ".n"] == n
    assert np.array_equal(f[name + ".colptr"], colptr)
    assert np.array_equal(f[name + ".rowval"], rowval)
    if exact:
        assert np.array_equal(f[name + ".nzval"].view(np.int64), nzval.view(np.int64))
    if ref is not None:
        _, _, rc, rr, rv = csc_fields(ref)
        assert np.array_equal(f[name + ".colptr"], rc) and np.array_equal(f[name + ".rowval"], rr)
        assert np.max(np.abs(f[name + ".nzval"] - rv)) <= 1e-13 * np.max(np.abs(rv))


@pytest.mark.parametrize("D,k,n", [(1, 2, 4), (2, 2, 3)])
def test_vlasov_h5_holds_the_reference_layout(sgdg, O, tmp_path, D, k, n):
    op = sgdg.VlasovOperator(D, k, n)
    P = 2 * D
    rng = np.random.default_rng(D * 10 + n)
    times = np.linspace(0.0, 0.25, 3)
    states = rng.standard_normal((3, op.N))
    path = str(tmp_path / "vlasov.h5")
    op.write_h5(path, times, states)
    f = read(path)
    names = {"dimensions", "order", "levels", "times"}
    for nm in list(WHICH) + ["Ds[%d]" % d for d in range(1, P + 1)]:
        names |= {nm + s for s in (".m", ".n", ".colptr", ".rowval", ".nzval")}
    names |= {"f_modal.%06d" % i for i in (1, 2, 3)}
    assert set(f) == names
    assert (f["dimensions"], f["order"], f["levels"]) == (D, k, n)
    assert f["dimensions"].dtype == np.int64 and f["times"].dtype == np.float64
    ops = O.vlasov_operators(D, k, n)
    for i, (nm, w) in enumerate(WHICH.items()):
        check_operator(f, nm, op.transform(*w), ref=ops[1 + i])
    for d in range(1, P + 1):
        check_operator(f, "Ds[%d]" % d, sgdg.D_matrix(P, d, k, n), ref=ops[0][d - 1])
    assert np.array_equal(f["times"], times)
    for i in range(3):
        assert np.array_equal(f["f_modal.%06d" % (i + 1)], states[i])
    op.close()


def test_vlasov_h5_operators_only_and_errors(sgdg, tmp_path):
    op = sgdg.VlasovOperator(1, 2, 3)
    path = str(tmp_path / "ops.h5")
    op.write_h5(path)
    f = read(path)
    assert "times" not in f and not any(k.startswith("f_modal") for k in f)
    assert len(f) == 3 + 5 * (4 + 2)
    # a directory that does not exist: SGDG_EIO
    with pytest.raises(sgdg.SGDGError) as e:
        op.write_h5(os.path.join(str(tmp_path), "no", "such", "dir.h5"))
    assert e.value.code == 8
    with pytest.raises(ValueError):
        op.write_h5(path, [0.0, 1.0], np.zeros((3, op.N)))
    op.close()


def test_h5_reader_rejects_a_damaged_file(sgdg, tmp_path):
    # the reader is strict: a changed byte in the structures fails a check
    op = sgdg.VlasovOperator(1, 2, 3)
    path = str(tmp_path / "ops.h5")
    op.write_h5(path)
    good = bytearray(open(path, "rb").read())
    for off in (0, 16, 40, 56 + 16):  # signature, leaf K, end of file, root cache type
        bad = bytearray(good)
        bad[off] ^= 0x5A
        open(path, "wb").write(bytes(bad))
        with pytest.raises(Exception):
            read(path)
    op.close()
