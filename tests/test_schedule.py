"""Level schedule of sparse ICD calls (mbir_level_schedule, host only, no GPU).

A level-scheduled bright-field NHICD call runs the call's voxel lines level by level; its result
equals the row walk's visit order when (1) lines of one level touch disjoint detector bins and
are not 3x3 (z, x) neighbours, and (2) along every bin and every neighbour pair the levels rise in
visit order.  These tests check both properties directly and compare the schedule with a Python
restatement of its definition."""
import numpy as np
import pytest


def footprints(n_z, n_x, n_r, tilts_deg, hw=1.0):
    """First bin and nonzero mask of a unit-voxel footprint per (z, x, view): bins
    [floor(u - hw), floor(u + hw)] inside the detector, u the projected voxel centre."""
    th = np.deg2rad(np.asarray(tilts_deg, np.float64))
    z = np.arange(n_z)[:, None, None] - n_z / 2 + 0.5
    x = np.arange(n_x)[None, :, None] - n_x / 2 + 0.5
    u = x * np.cos(th) - z * np.sin(th) + n_r / 2
    lo = np.floor(u - hw).astype(np.int64)
    hi = np.floor(u + hw).astype(np.int64)
    nb = int(2 * np.ceil(hw) + 1)
    mask = np.zeros(lo.shape, np.uint16)
    for b in range(nb):
        j = lo + b
        ok = (j <= hi) & (j >= 0) & (j < n_r)
        mask |= (ok.astype(np.uint16) << b)
    lo = np.where(mask != 0, lo, 0)
    return lo.astype(np.int16), mask, nb


def visit_order(rows, lineok, active, stride):
    n_z, n_x = lineok.shape
    out = []
    for z in rows:
        for k in range(min(stride, n_x)):
            for x in range(k, n_x, stride):
                if lineok[z, x] and (active is None or active[z, x]):
                    out.append(z * n_x + x)
    return out


def py_schedule(rows, lineok, active, lo, mask, nb, stride, n_r):
    """The schedule's definition, line by line."""
    n_z, n_x, n_t = lo.shape
    bin_level = np.zeros((n_t, n_r), np.int64)
    line_level = np.zeros((n_z, n_x), np.int64)
    order, levels = [], []
    for l in visit_order(rows, lineok, active, stride):
        z, x = divmod(l, n_x)
        m = 0
        for v in range(n_t):
            for b in range(nb):
                if (int(mask[z, x, v]) >> b) & 1:
                    m = max(m, bin_level[v, lo[z, x, v] + b])
        m = max(m, line_level[max(z - 1, 0):z + 2, max(x - 1, 0):x + 2].max())
        L = m + 1
        for v in range(n_t):
            for b in range(nb):
                if (int(mask[z, x, v]) >> b) & 1:
                    bin_level[v, lo[z, x, v] + b] = L
        line_level[z, x] = L
        order.append(l)
        levels.append(L)
    n_lev = max(levels) if levels else 0
    lines = [l for L in range(1, n_lev + 1) for l, q in zip(order, levels) if q == L]
    lofs = [0]
    for L in range(1, n_lev + 1):
        lofs.append(lofs[-1] + levels.count(L))
    return np.array(lines, np.int32), np.array(lofs, np.int32)


def check_schedule(lines, lofs, rows, lineok, active, lo, mask, nb, stride):
    """Properties (1) and (2) of the module docstring, O(lines x views)."""
    n_z, n_x, n_t = lo.shape
    order = visit_order(rows, lineok, active, stride)
    assert sorted(lines.tolist()) == sorted(order)
    level = {}
    for L in range(len(lofs) - 1):
        assert lofs[L + 1] > lofs[L], "empty level"
        for l in lines[lofs[L]:lofs[L + 1]]:
            level[int(l)] = L
    last_bin = {}
    last_line = np.full((n_z, n_x), -1, np.int64)
    for l in order:
        z, x = divmod(l, n_x)
        L = level[l]
        for v in range(n_t):
            for b in range(nb):
                if (int(mask[z, x, v]) >> b) & 1:
                    key = (v, int(lo[z, x, v]) + b)
                    if key in last_bin:
                        assert last_bin[key] < L, f"bin {key}: levels do not rise"
                    last_bin[key] = L
        nbh = last_line[max(z - 1, 0):z + 2, max(x - 1, 0):x + 2]
        assert (nbh < L).all(), "neighbour in the same or a later level"
        last_line[z, x] = L


def test_schedule_matches_definition_small(lib_built):
    mbir = lib_built
    rng = np.random.default_rng(11)
    n_z, n_x, n_r = 7, 24, 28
    lo, mask, nb = footprints(n_z, n_x, n_r, np.arange(-60, 61, 24))
    lineok = (rng.random((n_z, n_x)) < 0.9).astype(np.uint8)
    for frac, stride in ((1.0, 3), (0.3, 3), (0.05, 4)):
        active = (rng.random((n_z, n_x)) < frac).astype(np.uint8)
        rows = rng.permutation(n_z).astype(np.int32)
        lines, lofs = mbir.level_schedule(rows, lineok, lo, mask, nb, stride, n_r, active)
        pl, po = py_schedule(rows, lineok, active, lo, mask, nb, stride, n_r)
        np.testing.assert_array_equal(lines, pl)
        np.testing.assert_array_equal(lofs, po)
        check_schedule(lines, lofs, rows, lineok, active, lo, mask, nb, stride)


def test_schedule_bright_field_call_shape(lib_built):
    """A 1/20 NHICD call on a 64 x 256 plane with 61 views over +-60 deg: properties hold, and
    the call needs far fewer levels than the row walk has class steps."""
    mbir = lib_built
    rng = np.random.default_rng(5)
    n_z, n_x, n_r = 64, 256, 256
    lo, mask, nb = footprints(n_z, n_x, n_r, np.arange(-60, 61, 2))
    lineok = (mask != 0).any(axis=2).astype(np.uint8)
    active = np.zeros(n_z * n_x, np.uint8)
    active[rng.permutation(n_z * n_x)[: n_z * n_x // 20]] = 1
    active = active.reshape(n_z, n_x)
    rows = rng.permutation(n_z).astype(np.int32)
    stride = 6
    lines, lofs = mbir.level_schedule(rows, lineok, lo, mask, nb, stride, n_r, active)
    check_schedule(lines, lofs, rows, lineok, active, lo, mask, nb, stride)
    row_steps = sum(len({x % stride for x in np.nonzero(active[z] & lineok[z])[0]})
                    for z in range(n_z))
    assert len(lofs) - 1 < row_steps / 2


def test_schedule_all_lines_and_empty_call(lib_built):
    mbir = lib_built
    n_z, n_x, n_r = 5, 16, 20
    lo, mask, nb = footprints(n_z, n_x, n_r, [-30.0, 0.0, 30.0])
    lineok = np.ones((n_z, n_x), np.uint8)
    rows = np.arange(n_z, dtype=np.int32)
    lines, lofs = mbir.level_schedule(rows, lineok, lo, mask, nb, 3, n_r, None)
    check_schedule(lines, lofs, rows, lineok, None, lo, mask, nb, 3)
    lines, lofs = mbir.level_schedule(rows, lineok, lo, mask, nb, 3, n_r,
                                      np.zeros((n_z, n_x), np.uint8))
    assert lines.size == 0 and lofs.tolist() == [0]


def test_schedule_rejects_bad_input(lib_built):
    mbir = lib_built
    n_z, n_x, n_r = 4, 8, 10
    lo, mask, nb = footprints(n_z, n_x, n_r, [0.0, 20.0])
    lineok = np.ones((n_z, n_x), np.uint8)
    with pytest.raises(mbir.MbirError):   # row index out of range
        mbir.level_schedule(np.array([0, 1, 2, 9], np.int32), lineok, lo, mask, nb, 2, n_r)
    bad = mask.copy()
    bad[0, 0, 0] = 1 << 5                  # bit beyond nb
    with pytest.raises(mbir.MbirError):
        mbir.level_schedule(np.arange(n_z, dtype=np.int32), lineok, lo, bad, nb, 2, n_r)
    badlo = lo.copy()
    badlo[1, 1, 1] = n_r                  # touched bin past the detector
    with pytest.raises(mbir.MbirError):
        mbir.level_schedule(np.arange(n_z, dtype=np.int32), lineok, badlo, mask, nb, 2, n_r)


def py_colour(lineok, active, lo, mask, nb, cap=0):
    """Greedy colouring by definition: lines z-major, smallest colour no conflicting earlier
    line holds and with fewer than cap lines (cap 0: no limit)."""
    n_z, n_x, n_t = lo.shape
    col = {}
    bins = {}
    for z in range(n_z):
        for x in range(n_x):
            if not lineok[z, x] or (active is not None and not active[z, x]):
                continue
            used = set()
            mine = [(v, int(lo[z, x, v]) + b) for v in range(n_t) for b in range(nb)
                    if (int(mask[z, x, v]) >> b) & 1]
            for key in mine:
                used |= bins.get(key, set())
            for zz in range(max(z - 1, 0), min(z + 2, n_z)):
                for xx in range(max(x - 1, 0), min(x + 2, n_x)):
                    if (zz, xx) in col:
                        used.add(col[(zz, xx)])
            c = 0
            while c in used or (cap and sum(1 for q in col.values() if q == c) >= cap):
                c += 1
            col[(z, x)] = c
            for key in mine:
                bins.setdefault(key, set()).add(c)
    n = max(col.values()) + 1 if col else 0
    lines = [z * n_x + x for c in range(n) for (z, x), q in sorted(col.items()) if q == c]
    lofs = [0]
    for c in range(n):
        lofs.append(lofs[-1] + sum(1 for q in col.values() if q == c))
    return np.array(lines, np.int32), np.array(lofs, np.int32)


def check_independent(lines, lofs, lo, mask, nb):
    """No two lines of one colour class share a touched bin or are 3x3 (z, x) neighbours."""
    n_z, n_x, n_t = lo.shape
    for c in range(len(lofs) - 1):
        seen = {}
        pos = set()
        for l in lines[lofs[c]:lofs[c + 1]]:
            z, x = divmod(int(l), n_x)
            for zz in range(z - 1, z + 2):
                for xx in range(x - 1, x + 2):
                    assert (zz, xx) not in pos, f"colour {c}: neighbours {(z, x)}, {(zz, xx)}"
            pos.add((z, x))
            for v in range(n_t):
                for b in range(nb):
                    if (int(mask[z, x, v]) >> b) & 1:
                        key = (v, int(lo[z, x, v]) + b)
                        assert key not in seen, f"colour {c}: bin {key} shared"
                        seen[key] = l


def test_colour_schedule_matches_definition(lib_built):
    mbir = lib_built
    rng = np.random.default_rng(12)
    n_z, n_x, n_r = 7, 24, 28
    lo, mask, nb = footprints(n_z, n_x, n_r, np.arange(-60, 61, 24))
    lineok = (rng.random((n_z, n_x)) < 0.9).astype(np.uint8)
    for frac, cap in ((1.0, 0), (0.3, 0), (0.05, 0), (1.0, 3), (0.3, 2)):
        active = (rng.random((n_z, n_x)) < frac).astype(np.uint8)
        lines, lofs = mbir.colour_schedule(lineok, lo, mask, nb, n_r, active, class_cap=cap)
        pl, po = py_colour(lineok, active, lo, mask, nb, cap)
        np.testing.assert_array_equal(lines, pl)
        np.testing.assert_array_equal(lofs, po)
        check_independent(lines, lofs, lo, mask, nb)
        if cap:
            assert np.diff(lofs).max() <= cap


def test_colour_schedule_bright_field_call_shape(lib_built):
    """A 1/20 NHICD call on a 64 x 256 plane, 61 views over +-60 deg: every class independent,
    every line once, and fewer classes than the row walk's dependency levels."""
    mbir = lib_built
    rng = np.random.default_rng(5)
    n_z, n_x, n_r = 64, 256, 256
    lo, mask, nb = footprints(n_z, n_x, n_r, np.arange(-60, 61, 2))
    lineok = (mask != 0).any(axis=2).astype(np.uint8)
    active = np.zeros(n_z * n_x, np.uint8)
    active[rng.permutation(n_z * n_x)[: n_z * n_x // 20]] = 1
    active = active.reshape(n_z, n_x)
    lines, lofs = mbir.colour_schedule(lineok, lo, mask, nb, n_r, active)
    check_independent(lines, lofs, lo, mask, nb)
    assert sorted(lines.tolist()) == sorted(np.flatnonzero(active & lineok).tolist())
    rows = rng.permutation(n_z).astype(np.int32)
    _, lvl = mbir.level_schedule(rows, lineok, lo, mask, nb, 6, n_r, active)
    assert len(lofs) < len(lvl)
    capped, cofs = mbir.colour_schedule(lineok, lo, mask, nb, n_r, active, class_cap=16)
    check_independent(capped, cofs, lo, mask, nb)
    assert np.diff(cofs).max() <= 16 and sorted(capped.tolist()) == sorted(lines.tolist())
    with pytest.raises(mbir.MbirError):  # more colours needed than allowed
        mbir.colour_schedule(lineok, lo, mask, nb, n_r, active, max_colours=4)
