"""The matrix-free work list, built on the host by the dry run of the C ABI
(no GPU): the schedule can never deadlock (every counter an item waits for
is incremented only by items earlier in the list, and its target is their
count), the stages of a whole-step list follow each other per group, and
the tiles' index arithmetic -- restated here from the stage kernel's column
decode, row table and invariant-divisor division -- covers every element
of every solve exactly once per phase and stays inside the solve."""
import ctypes

import numpy as np
import pytest

TILE_FIRST, TILE_LAST, TILE_RK, TILE_STORE, TILE_WACC, TILE_WAIT_IN, TILE_SUMIN = 1, 2, 4, 8, 16, 32, 64
FIELDS = ["cls", "d", "tab", "flags", "src", "dst", "wsel", "stage", "wait_ctr", "wait_need", "win_ctr",
          "win_need", "done_ctr", "lmax", "lp", "boff", "R", "g0", "W", "Wv", "kd1", "kDm1", "rlong", "rmagic",
          "rshift"]
ADVECT, WAVE, VLASOV = 0, 1, 2


def dryrun(sgdg, classes, pass_only=False, chunk=0, nchunks=1):
    """classes: (kind, D, k, n, scheme, solves, apply, apply_dim) per class."""
    L = sgdg.lib()
    spec = np.ascontiguousarray(np.array(classes, dtype=np.int32).reshape(-1, 8))
    ni, nb, nc = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
    args = (len(spec), spec.ctypes.data, int(pass_only), chunk, nchunks)
    assert L.sgdg_worklist_dryrun(*args, None, 0, ctypes.byref(ni), ctypes.byref(nc), None, None, 0,
                                  ctypes.byref(nb)) == 0
    items = np.zeros((ni.value, len(FIELDS)), dtype=np.int64)
    boff = np.zeros(max(nb.value, 1), dtype=np.int64)
    cls = np.zeros((len(spec), 4), dtype=np.int64)
    assert L.sgdg_worklist_dryrun(*args, items.ctypes.data, ni.value, ctypes.byref(ni), ctypes.byref(nc),
                                  cls.ctypes.data, boff.ctypes.data, nb.value, ctypes.byref(nb)) == 0
    it = {f: items[:, i] for i, f in enumerate(FIELDS)}
    return it, spec, cls, boff, nc.value


def tile_elements(it, i, spec_c, cls_c, boff):
    """(slot, element offset) of every valid element of item i, as the stage kernel addresses them."""
    K, D = int(spec_c[2]), int(spec_c[1])
    kD = K ** D
    R, g0, Wv, lp, lmax = (int(it[f][i]) for f in ("R", "g0", "Wv", "lp", "lmax"))
    kd1, kDm1, bo = int(it["kd1"][i]), int(it["kDm1"][i]), int(it["boff"][i])
    g = g0 + np.arange(Wv, dtype=np.int64)
    # the kernel's division by the invariant R: (g * magic) >> shift
    slot = (g.astype(np.uint64) * np.uint64(it["rmagic"][i])) >> np.uint64(it["rshift"][i])
    slot = slot.astype(np.int64)
    assert np.array_equal(slot, g // R)
    r = g - slot * R
    cr = r // kDm1
    mr = r - cr * kDm1
    mq = mr // kd1
    ca = kD * (cr & ((1 << lp) - 1)) + (mr - mq * kd1) + mq * kd1 * K
    cb = kD * ((cr >> lp) << lp)
    m = K << (lmax - 1)
    row = np.arange(m, dtype=np.int64)
    rb = row // K
    md = row - rb * K
    lev = np.where(rb == 0, 1, np.floor(np.log2(np.maximum(rb, 1))).astype(np.int64) + 2)
    cd0 = np.where(lev >= 2, rb - (1 << np.maximum(lev - 2, 0)), 0)
    first = int(cls_c[3])
    rx = boff[first + bo + lev - 1] + kD * (cd0 << lp) + md * kd1
    ry = np.maximum(lev - 2, 0)
    off = rx[:, None] + (cb[None, :] << ry[:, None]) + ca[None, :]
    return np.broadcast_to(slot[None, :], off.shape).ravel(), off.ravel()


def check_schedule(it, nctr):
    n = len(it["cls"])
    done = it["done_ctr"]
    assert done.min() >= 1 and done.max() < nctr  # counter 0 hands out the items
    last = np.full(nctr, -1)
    count = np.zeros(nctr, dtype=np.int64)
    np.maximum.at(last, done, np.arange(n))
    np.add.at(count, done, 1)
    for key, need in (("wait_ctr", "wait_need"), ("win_ctr", "win_need")):
        c = it[key]
        has = c > 0
        idx = np.nonzero(has)[0]
        # every incrementing item comes earlier in the list, and the target is their number
        assert np.all(last[c[has]] < idx), key
        assert np.array_equal(it[need][has], count[c[has]]), key


def check_coverage(it, spec, cls, boff):
    """Every phase (the items sharing a counter, dimension and vectors; the
    wave's short and long lines of one phase use different tables) covers
    each element of each of its group's solves exactly once."""
    n = len(it["cls"])
    keys = np.stack([it["done_ctr"], it["d"], it["src"], it["dst"], it["wsel"], it["stage"]], axis=1)
    phases = {}
    for i in range(n):
        phases.setdefault(tuple(keys[i]), []).append(i)
    for members in phases.values():
        c = int(it["cls"][members[0]])
        N = int(cls[c][0])
        slots, offs = [], []
        for i in members:
            assert it["cls"][i] == c
            s, o = tile_elements(it, i, spec[c], cls[c], boff)
            slots.append(s)
            offs.append(o)
        s, o = np.concatenate(slots), np.concatenate(offs)
        assert o.min() >= 0 and o.max() < N  # inside the solve (the debug build's check)
        lo, hi = s.min(), s.max()
        hits = np.bincount((s - lo) * N + o, minlength=(hi - lo + 1) * N)
        assert np.all(hits == 1), (c, len(members))
    return phases


def group_slots(it, i):
    g0, Wv, R = int(it["g0"][i]), int(it["Wv"][i]), int(it["R"][i])
    return g0 // R, (g0 + Wv - 1) // R


def check_stages(it):
    """Whole-step lists: four stages; every stage-input gather of stages 2-4
    waits for the RK phase of the previous stage over the same solves."""
    n = len(it["cls"])
    stepping = np.nonzero(it["stage"] > 0)[0]
    if len(stepping) == 0:
        assert np.all(it["win_ctr"] <= 0)
        return
    assert set(it["stage"][stepping].tolist()) == {1, 2, 3, 4}
    rk_of = {}
    for i in stepping:
        if it["flags"][i] & TILE_RK:
            rk_of.setdefault(int(it["done_ctr"][i]), []).append(i)
    for i in stepping:
        st = it["stage"][i]
        gathers = it["src"][i] < 0
        if st == 1 or not gathers:
            assert it["win_ctr"][i] <= 0
            continue
        c = int(it["win_ctr"][i])
        assert c in rk_of
        prev = rk_of[c]
        assert all(it["stage"][j] == st - 1 and it["cls"][j] == it["cls"][i] for j in prev)
        lo = min(group_slots(it, j)[0] for j in prev)
        hi = max(group_slots(it, j)[1] for j in prev)
        a, b = group_slots(it, i)
        assert lo <= a and b <= hi


def check_rk_once(it, spec, cls, boff):
    """Per class and stage, the RK phases together update every element once."""
    rk = np.nonzero((it["flags"] & TILE_RK) != 0)[0]
    for c in range(len(spec)):
        for st in (1, 2, 3, 4):
            sel = [i for i in rk if it["cls"][i] == c and it["stage"][i] == st]
            if not sel:
                continue
            N, ns = int(cls[c][0]), int(cls[c][2])
            hits = np.zeros(ns * N, dtype=np.int64)
            for i in sel:
                s, o = tile_elements(it, i, spec[c], cls[c], boff)
                np.add.at(hits, s * N + o, 1)
            assert np.all(hits == 1), (c, st)


BATCHES = [
    # one wave class (the bench's kind, smaller), whole RK4 step
    [(WAVE, 3, 3, 4, 0, 5, 0, 0)],
    # uneven classes in one list
    [(ADVECT, 2, 2, 5, 0, 7, 0, 0), (WAVE, 2, 4, 4, 0, 3, 0, 0), (ADVECT, 3, 5, 3, 0, 2, 0, 0)],
    # the full scheme, one dimension
    [(ADVECT, 2, 2, 3, 1, 4, 0, 0), (WAVE, 1, 3, 6, 0, 2, 0, 0)],
    # operator applications: the sum over dimensions and one dimension
    [(ADVECT, 3, 2, 4, 0, 3, 1, -1), (ADVECT, 3, 2, 4, 0, 2, 1, 1)],
    # Vlasov 2x2v: the transform chains and their join
    [(VLASOV, 4, 2, 3, 0, 2, 0, 0)],
]


@pytest.mark.parametrize("batch", range(len(BATCHES)))
def test_worklist_schedule_and_tiles(sgdg, batch):
    it, spec, cls, boff, nctr = dryrun(sgdg, BATCHES[batch])
    assert len(it["cls"]) > 0
    check_schedule(it, nctr)
    check_coverage(it, spec, cls, boff)
    check_stages(it)
    check_rk_once(it, spec, cls, boff)


def test_worklist_pass_only_list(sgdg):
    it, spec, cls, boff, nctr = dryrun(sgdg, BATCHES[0], pass_only=True)
    check_schedule(it, nctr)
    check_coverage(it, spec, cls, boff)
    assert np.all(it["stage"] == 0) and not np.any(it["flags"] & TILE_RK)
    assert sorted(set(it["d"].tolist())) == [0, 1, 2]


@pytest.mark.parametrize("wlog,coop", [(-2, 1), (-1, 3), (1, 5), (3, 30)])
def test_worklist_tile_shapes(sgdg, wlog, coop):
    try:
        sgdg.set_tile_shape(3, 3, wlog, coop)
        it, spec, cls, boff, nctr = dryrun(sgdg, BATCHES[0])
        check_schedule(it, nctr)
        check_coverage(it, spec, cls, boff)
        check_rk_once(it, spec, cls, boff)
        # wider tiles, fewer items
        assert np.all(it["W"] % 4 == 0) and np.all(it["Wv"] <= it["W"])
    finally:
        sgdg.clear_tile_shapes()


def test_worklist_dryrun_rejects_bad_specs(sgdg):
    L = sgdg.lib()
    ni, nb = ctypes.c_int64(), ctypes.c_int64()
    for bad in ([(7, 2, 2, 3, 0, 1, 0, 0)], [(ADVECT, 2, 9, 3, 0, 1, 0, 0)], [(ADVECT, 2, 2, 3, 0, 0, 0, 0)],
                [(VLASOV, 3, 2, 3, 0, 1, 0, 0)], [(ADVECT, 2, 2, 3, 0, 1, 1, 5)]):
        spec = np.ascontiguousarray(np.array(bad, dtype=np.int32).reshape(-1, 8))
        code = L.sgdg_worklist_dryrun(1, spec.ctypes.data, 0, 0, 1, None, 0, ctypes.byref(ni), None, None, None, 0,
                                      ctypes.byref(nb))
        assert code != 0, bad


@pytest.mark.parametrize("nchunks", [2, 3, 16])
def test_worklist_pipeline_chunks(sgdg, nchunks):
    """The host-to-host step's chunk lists: each is a valid schedule of its
    own, and together they update every element of every solve once per
    stage (each class's groups are cut into nchunks runs)."""
    # 100 wave solves of 18,576 coefficients per component: groups of 42 solves
    # (6 MB of stage input and partial sums each), so the chunks hold groups
    batch = [(WAVE, 3, 3, 6, 0, 100, 0, 0), (ADVECT, 2, 2, 3, 0, 9, 0, 0)]
    hits = None
    nonempty = 0
    for ch in range(nchunks):
        it, spec, cls, boff, nctr = dryrun(sgdg, batch, chunk=ch, nchunks=nchunks)
        if hits is None:
            hits = {(c, st): np.zeros(int(cls[c][2] * cls[c][0]), dtype=np.int64)
                    for c in range(len(spec)) for st in (1, 2, 3, 4)}
        if len(it["cls"]) == 0:
            continue
        nonempty += 1
        check_schedule(it, nctr)
        check_coverage(it, spec, cls, boff)
        check_stages(it)
        for i in np.nonzero((it["flags"] & TILE_RK) != 0)[0]:
            c = int(it["cls"][i])
            s, o = tile_elements(it, i, spec[c], cls[c], boff)
            np.add.at(hits[(c, int(it["stage"][i]))], s * int(cls[c][0]) + o, 1)
    for key, h in hits.items():
        assert np.all(h == 1), key
    assert nonempty == min(nchunks, 3)  # the wave class's three groups, the advection class's one


def test_worklist_groups(sgdg):
    it, spec, cls, boff, nctr = dryrun(sgdg, [(WAVE, 3, 3, 6, 0, 100, 0, 0)])
    firsts = sorted({int(it["done_ctr"][i]) for i in range(len(it["cls"]))})
    assert len(firsts) == nctr - 1
