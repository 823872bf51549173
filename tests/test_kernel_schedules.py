"""Index arithmetic of the FP32 kernels' reverse windows, replayed on the CPU:
the two-threads-per-path kernel (csrc/lmm_f32_tp2.cu) for NN=160, NMAT=120,
and the thread-per-path kernel (csrc/lmm_f32_tpp.cu) for NN=80, NMAT=40.

The kernel splits a path's rates between a lower and an upper warp and runs
the reverse sweep in barrier-separated rounds: in round r the upper half takes
the step group r and the lower half the group r-1. Each half accumulates vega
rows of one shared per-path table without atomics, which is correct only if
the rows the two halves touch in one round are disjoint. These tests enumerate
every round with the kernel's own window rules (chunked positions, the early
exit below the lowest active cell, ring flush slots, the final flush of slot 0)
and check that, and that every constant and vega row the windows address lies
inside the shared-memory tables (constant rows >= -NMAT, vega rows >= -16).
"""
import pytest

NN, NMAT, H = 160, 120, 80
CH, P, G = 8, 2, 2          # chunk, constant prefetch distance, steps per group
VPAD, PADK = 16, NMAT       # spare vega rows, zero constant rows in front


def rev_window(base, n):
    """Vega rows (as k) flushed and constant rows (as k) loaded by the reverse
    window of steps n, n-1 over the half whose first global rate is base."""
    jmax = H + G - 2
    imin = n - 1 - base
    slots, consts = set(), set()
    if imin >= H:                       # the kernel skips a half with no active cell
        return set(), set()
    consts.update(range(H - P, jmax + 1))
    completed = True
    q = 0
    while q * CH < H + G - 1:
        top = H - 1 - q * CH
        if top < imin:
            completed = False
            break
        i = top
        while i > top - CH and i >= -(G - 1):
            if i - P >= 0:
                consts.add(i - P)
            jf = i + 2 * (G - 1)
            if 0 <= jf <= jmax:
                slots.add(jf)
            i -= 1
        q += 1
    if completed:
        slots.add(0)
    to_k = lambda j: base + j - n - 1
    return {to_k(j) for j in slots}, {to_k(j) for j in consts}


def fwd_window_consts(base, n):
    """Constant rows (as k) loaded by the forward window of steps n, n+1."""
    first = n + 1 - base
    if first >= H:
        return set()
    c0 = first // CH if first > 0 else 0
    consts = {j for j in range(c0 * CH - 2, c0 * CH + P) if j < H}
    for c in range(c0, H // CH):
        for p in range(c * CH, (c + 1) * CH):
            if p + P < H:
                consts.add(p + P)
    return {base + j - n - 1 for j in consts}


def test_reverse_rounds_touch_disjoint_vega_rows():
    for r in range(NMAT // 2 + 1):
        up_rows = low_rows = set()
        if r < NMAT // 2:
            up_rows, _ = rev_window(H, NMAT - 1 - 2 * r)
        if r >= 1:
            low_rows, _ = rev_window(0, NMAT - 1 - 2 * (r - 1))
        assert not (up_rows & low_rows), (r, sorted(up_rows & low_rows))


@pytest.mark.parametrize("base", [0, H])
def test_windows_stay_inside_the_tables(base):
    for n in range(NMAT - 1, 0, -2):
        rows, consts = rev_window(base, n)
        assert all(-VPAD <= k <= NN - 1 for k in rows), (base, n, min(rows), max(rows))
        assert all(-PADK <= k <= NN - 1 for k in consts), (base, n)
    for n in range(0, NMAT, 2):
        consts = fwd_window_consts(base, n)
        assert all(-PADK <= k <= NN - 1 for k in consts), (base, n)


def test_every_active_reverse_cell_is_flushed_to_its_own_row():
    """Each active cell (n', i) of a group adds to row k = i - n' - 1 of its
    own step; the flushed rows of the two halves together cover all of them."""
    for g in range(NMAT // 2):
        n = NMAT - 1 - 2 * g
        flushed = rev_window(H, n)[0] | rev_window(0, n)[0]
        for step in (n, n - 1):
            for i in range(step + 1, NN):
                assert i - step - 1 in flushed, (n, step, i)


def test_forward_hand_over_matches_the_steps_each_half_runs():
    """Forward round r: the lower half writes the drift sums of steps 2r, 2r+1
    into buffer r % 2; the upper half reads buffer (r-1) % 2 for steps 2r-2,
    2r-1, i.e. exactly what the lower half wrote one round earlier, before the
    lower half overwrites that buffer in round r+1."""
    written = {}
    for r in range(NMAT // 2 + 1):
        if r >= 1:
            assert written[(r - 1) % 2] == (2 * r - 2, 2 * r - 1)
        if r < NMAT // 2:
            written[r % 2] = (2 * r, 2 * r + 1)


# The fused two-threads-per-path kernel cuts the rates into blocks of L and
# the two roles own alternate blocks; block s runs forward steps 2(r-s),
# 2(r-s)+1 in round r and reverse steps n, n-1 with n = NMAT-1-2(r-(S-1-s)).
# The window rules per block are those above with the block's L rates and a
# chunk of 8 rates (4 when L is not a multiple of 8).
def blk_rev_window(L, lo, n):
    """Vega rows (as k) flushed and constant rows (as k) loaded by the reverse
    window of steps n, n-1 over the block of L rates from rate lo."""
    ch = 8 if L % 8 == 0 else 4
    jmax = L + G - 2
    imin = n - 1 - lo
    slots, consts = set(), set()
    if imin >= L:
        return set(), set()
    consts.update(range(L - P, jmax + 1))
    completed = True
    q = 0
    while q * ch < L + G - 1:
        top = L - 1 - q * ch
        if top < imin:
            completed = False
            break
        i = top
        while i > top - ch and i >= -(G - 1):
            if i - P >= 0:
                consts.add(i - P)
            jf = i + 2 * (G - 1)
            if 0 <= jf <= jmax:
                slots.add(jf)
            i -= 1
        q += 1
    if completed:
        slots.add(0)
    to_k = lambda j: lo + j - n - 1
    return {to_k(j) for j in slots}, {to_k(j) for j in consts}


@pytest.mark.parametrize("L", [80, 40, 20])
def test_block_rounds_touch_disjoint_vega_rows_and_stay_in_the_tables(L):
    """In every reverse round the rows the blocks flush are pairwise disjoint
    between the two roles' blocks (each role runs its own blocks one after
    another), and every row and constant lies inside the tables."""
    S = NN // L
    for r in range(NMAT // 2 + S - 1):
        per_role = {0: [], 1: []}
        for s in range(S):
            jr = r - (S - 1 - s)
            if not 0 <= jr < NMAT // 2:
                continue
            n = NMAT - 1 - 2 * jr
            rows, consts = blk_rev_window(L, s * L, n)
            assert all(-VPAD <= k <= NN - 1 for k in rows), (L, r, s, min(rows))
            assert all(-PADK <= k <= NN - 1 for k in consts), (L, r, s)
            per_role[s % 2].append(rows)
        a = set().union(*per_role[0]) if per_role[0] else set()
        b = set().union(*per_role[1]) if per_role[1] else set()
        assert not (a & b), (L, r, sorted(a & b))


@pytest.mark.parametrize("L", [80, 40, 20])
def test_block_reverse_flushes_every_active_cell(L):
    """Each active cell (n', i) adds to row k = i - n' - 1: the block holding
    rate i, in the round it runs step n', flushes that row."""
    S = NN // L
    for s in range(S):
        for jr in range(NMAT // 2):
            n = NMAT - 1 - 2 * jr
            rows, _ = blk_rev_window(L, s * L, n)
            for step in (n, n - 1):
                for i in range(max(step + 1, s * L), (s + 1) * L):
                    assert i - step - 1 in rows, (L, s, n, step, i)


@pytest.mark.parametrize("L", [80, 40, 20])
def test_block_hand_overs_match_the_steps_each_block_runs(L):
    """Forward: block s reads in round r the buffer (s-1, (r-1) % 2) that block
    s-1 wrote in round r-1 for the same steps, and block s-1 writes that
    buffer again only in round r+1. Reverse: the same downwards."""
    S = NN // L
    fw, rv = {}, {}
    for r in range(NMAT // 2 + S - 1):
        for s in range(S):
            n = 2 * (r - s)
            if 0 <= n < NMAT:
                if s > 0:
                    assert fw[(s - 1, (r - 1) % 2)] == (r - 1, n), (L, r, s)
                if s < S - 1:
                    fw[(s, r % 2)] = (r, n)
            jr = r - (S - 1 - s)
            if 0 <= jr < NMAT // 2:
                n = NMAT - 1 - 2 * jr
                if s < S - 1:
                    assert rv[(s, (r - 1) % 2)] == (r - 1, n), (L, r, s)
                if s > 0:
                    rv[(s - 1, r % 2)] = (r, n)


# The thread-per-path kernel (csrc/lmm_f32_tpp.cu) leaves its reverse body
# early in the same way: a group of G steps n, n-1, ..., n-G+1 runs positions
# from the top in chunks and returns at the first chunk wholly below its
# lowest active position n - 2G + 3; a vega slot j is flushed (row k = j-n-1)
# at position j - 2(G-1). Settings as built: fused G = 4 with 2-rate chunks
# (4 with Philox normals), backward-only G = 2 with 2-rate chunks.
TPP_NN, TPP_NMAT, TPP_PAD = 80, 40, 40
TPP_VPAD = 4                # spare vega rows in front of row 0 (lmm_f32_tpp.cu TppLayout::VPAD)


def tpp_rev_window(n, G, ch, p):
    jmax = TPP_NN + G - 2
    imin = n - 2 * G + 3
    flushed, consts = set(), set(range(TPP_NN - p, jmax + 1))
    q = 0
    while q * ch < TPP_NN + G - 1:
        top = TPP_NN - 1 - q * ch
        if top < imin:
            break
        i = top
        while i > top - ch and i >= -(G - 1):
            if i - p >= 1:
                consts.add(i - p)
            jf = i + 2 * (G - 1)
            if 1 <= jf <= jmax:
                flushed.add(jf)
            i -= 1
        q += 1
    return {j - n - 1 for j in flushed}, {j - n - 1 for j in consts}


@pytest.mark.parametrize("G,ch,p", [(4, 2, 1), (4, 4, 0), (2, 2, 1)])
def test_thread_per_path_reverse_windows(G, ch, p):
    for n in range(TPP_NMAT - 1, 0, -G):
        rows, consts = tpp_rev_window(n, G, ch, p)
        assert all(-TPP_VPAD <= k <= TPP_NN - 1 for k in rows), (n, min(rows))
        assert all(-TPP_PAD <= k <= TPP_NN - 1 for k in consts), (n, min(consts))
        for g in range(G):
            step = n - g
            for i in range(step + 1, TPP_NN):
                assert i - step - 1 in rows, (G, ch, n, step, i)


def half_window(n, G, ch, p, H, lo, nn=TPP_NN):
    """Replays rev_half_window (csrc/lmm_f32_tpp.cu, k_tps) for steps n..n-G+1
    over rates lo..lo+H-1: returns the flushes as (row k, set of cells) and
    the constant rows (as k) loaded. A cell is (step, rate)."""
    W = 2 * G - 1 + p
    jmax = H + G - 2
    low = 0 if lo > 0 else 1
    slots = {}
    flushes, consts = [], set(range(H - p, jmax + 1))
    for j in range(H, jmax + 1):
        slots[j % W] = (j, set())
    imin = n - 2 * G + 3 - lo
    q = 0
    while q * ch < H + G - 1:
        top = H - 1 - q * ch
        if lo == 0 and top < imin:
            return flushes, {lo + j - n - 1 for j in consts}
        i = top
        while i > top - ch and i >= -(G - 1):
            if i - p >= low:
                consts.add(i - p)
            if i >= low:
                slots[i % W] = (i, set())
            for g in range(G):
                if low <= i + g <= H - 1:
                    j = i + 2 * g
                    sj, cells = slots[j % W]
                    assert sj == j, (n, i, g, sj, j)          # the slot holds this j
                    cells.add((n - g, lo + i + g))
            jf = i + 2 * (G - 1)
            if low <= jf <= jmax:
                sj, cells = slots[jf % W]
                assert sj == jf
                flushes.append((lo + jf - n - 1, set(cells)))
            i -= 1
        q += 1
    if lo > 0:
        for j in range(G - 1):
            sj, cells = slots[j % W]
            assert sj == j
            flushes.append((lo + j - n - 1, set(cells)))
    return flushes, {lo + j - n - 1 for j in consts}


@pytest.mark.parametrize("ch", [1, 2, 4])
def test_split_reverse_half_windows(ch):
    """k_tps: the upper half (rates 40..79) and then the lower half (rates
    0..39) over every group of four steps flush every active cell's vega
    contribution exactly once, to the row k = rate - step - 1 of its own
    step; rows with active cells lie in 0..NN-1, spare rows in -VPAD..-1, and
    every constant row loaded in -NMAT..NN-1."""
    G, p, H = 4, 1, TPP_NN // 2
    seen = {}
    for lo in (H, 0):
        for n in range(TPP_NMAT - 1, 0, -G):
            flushes, consts = half_window(n, G, ch, p, H, lo)
            assert all(-TPP_PAD <= k <= TPP_NN - 1 for k in consts), (lo, n)
            for k, cells in flushes:
                assert -TPP_VPAD <= k <= TPP_NN - 1, (lo, n, k)
                for step, rate in cells:
                    if rate > step:                      # active cell
                        assert k == rate - step - 1, (lo, n, step, rate, k)
                        seen[(step, rate)] = seen.get((step, rate), 0) + 1
    for step in range(TPP_NMAT):
        for rate in range(step + 1, TPP_NN):
            assert seen.get((step, rate)) == 1, (step, rate, seen.get((step, rate)))


def block_window(n, G, ch, p, H, lo, tl=None):
    """Replays rev_block_window (csrc/lmm_f32_tpp.cu, k_tpq): steps n..n-G+1
    over rates lo..lo+H-1 with the block's offset at run time. Returns the
    flushes as (row k, set of cells) and the constant rows (as k) loaded.
    With tl given, also checks the in-body loads of the rates the caller
    replaces (local positions j > tl): each comes after the group's last
    cell on its rate, and every such position is loaded once."""
    W = 2 * G - 1 + p
    jmax = H + G - 2
    full = lo > n
    slots = {}
    flushes, consts = [], set(range(H - p, jmax + 1))
    for j in range(H, jmax + 1):
        slots[j % W] = (j, set())
    imin = n - 2 * G + 3 - lo
    loaded = set()

    def done():
        if tl is not None:
            assert loaded == set(range(max(tl + 1, 0), H)), (lo, n, tl, sorted(loaded))
        return flushes, {lo + j - n - 1 for j in consts}

    q = 0
    while q * ch < H + G - 1:
        top = H - 1 - q * ch
        if not full and top < imin:
            return done()
        i = top
        while i > top - ch and i >= -(G - 1):
            if i - p >= 0:
                consts.add(i - p)
            if i >= 0:
                slots[i % W] = (i, set())
            for g in range(G):
                if 0 <= i + g <= H - 1:
                    j = i + 2 * g
                    sj, cells = slots[j % W]
                    assert sj == j, (lo, n, i, g, sj, j)
                    cells.add((n - g, lo + i + g))
                    assert i + g not in loaded, (lo, n, i, g)   # no cell after the rate's load
            jf = i + 2 * (G - 1)
            if 0 <= jf <= jmax:
                sj, cells = slots[jf % W]
                assert sj == jf
                flushes.append((lo + jf - n - 1, set(cells)))
            jr = i + G - 1
            if tl is not None and 0 <= jr <= H - 1 and jr > tl:
                assert jr not in loaded
                loaded.add(jr)
            i -= 1
        q += 1
    if full:
        for j in range(G - 1):
            sj, cells = slots[j % W]
            assert sj == j
            flushes.append((lo + j - n - 1, set(cells)))
    return done()


@pytest.mark.parametrize("G", [4, 8])
@pytest.mark.parametrize("ch", [2, 4])
def test_long_tenor_block_passes(ch, G):
    """k_tpq at NN=160, NMAT=120: the blocks of 40 rates from the top, each
    over its groups of G steps from the first group with an active cell,
    flush every active cell exactly once to its own row; every row lies in
    -VPAD..NN-1 and every constant row in -NMAT..NN-1; the groups a block skips
    have no active cell in it, and the block below skips them too (so it never
    reads a suffix sum the block above did not leave)."""
    NN, NMAT, p, H, VP = 160, 120, 1, 40, 4
    seen = {}
    first = {}
    for b in range(NN // H - 1, -1, -1):
        lo = b * H
        n0 = NMAT - 1
        while lo + H - 1 <= n0 - G + 1:
            n0 -= G
        first[b] = n0
        for n in range(NMAT - 1, n0, -G):           # skipped groups: no active cell in the block
            assert all(r <= m for m in range(n - G + 1, n + 1) for r in range(lo, lo + H))
        for n in range(n0, 0, -G):
            flushes, consts = block_window(n, G, ch, p, H, lo)
            assert all(-NMAT <= k <= NN - 1 for k in consts), (lo, n)
            for k, cells in flushes:
                assert -VP <= k <= NN - 1, (lo, n, k)
                for step, rate in cells:
                    if rate > step:
                        assert k == rate - step - 1, (lo, n, step, rate, k)
                        seen[(step, rate)] = seen.get((step, rate), 0) + 1
    for b in range(1, NN // H):
        assert first[b - 1] <= first[b]
    for step in range(NMAT):
        for rate in range(step + 1, NN):
            assert seen.get((step, rate)) == 1, (step, rate, seen.get((step, rate)))


@pytest.mark.parametrize("ck", [0, 4, 8, 12, 16, 40, 116])
@pytest.mark.parametrize("ch,G", [(2, 4), (4, 4), (2, 8), (4, 8)])
def test_long_tenor_checkpoints_and_hand_on_loads(ck, ch, G):
    """k_tpq's rate checkpoints every ck steps (ck a multiple of 4; 0: none)
    and the rates each group loads for the next: the forward saves
    checkpoint c after step (c+1)ck - 1 for the rates above (c+1)ck; a group
    ending at a checkpoint time t loads, inside its body and after its last
    cell on each, the block's rates above t from that checkpoint, only rates
    the forward saved and rows inside the scratch; a block's last group
    loads all of the parked rates of the block below, and no group has both
    loads."""
    NN, NMAT, H, p = 160, 120, 40, 1
    nck = (NMAT - 1) // ck if ck else 0
    ckd = ck if ck else 1
    saved = set()
    for n in range(0, NMAT, 2):
        if nck > 0 and (n + 2) % ckd == 0 and n + 2 < NMAT:
            c = (n + 2) // ckd - 1
            assert 0 <= c < nck
            saved |= {(c, i) for i in range(NN) if i > n + 2}
    for b in range(NN // H - 1, -1, -1):
        lo = b * H
        n0 = NMAT - 1
        while lo + H - 1 <= n0 - G + 1:
            n0 -= G
        parked = 0
        for n in range(n0, 0, -G):
            t = n - G + 1
            tl = H
            if nck > 0 and t % ckd == 0 and t >= ck:
                c = t // ckd - 1
                assert 0 <= c < nck and 0 <= c * NN + lo and c * NN + lo + H <= nck * NN
                tl = t - lo
                assert all((c, lo + j) in saved for j in range(max(tl + 1, 0), H)), (b, n, c)
                assert not (b > 0 and n - G <= 0)
            elif b > 0 and n - G <= 0:
                tl = -1
                parked += 1
                assert lo > n                    # a full window: every position is loaded
            block_window(n, G, ch, p, H, lo, tl)
        assert parked == (1 if b > 0 else 0), b


def fwd_pair_pass(NP, H, CH, P, LO, n, NMAT, NN, done):
    """Replays fwd_pair_pass (csrc/lmm_f32_tpp.cu, k_tpq's forward passes):
    steps n, n+1 over rates LO .. LO+NP-1. `done` maps a step to the rates
    whose cells it has run (active or not), in order; the constant of every
    cell must be its own k = rate - step - 1 and lie in the table
    (-NMAT .. NN-1). Returns, per step, the rates summed into V0c/V1c[q]."""
    R = 3 + P
    C = {}
    nrel = n - LO
    c0 = (nrel + 1) // CH if nrel + 1 > 0 else 0
    # V0c/V1c start as the entering sums (no cell of the pass yet)
    caps = {st: [list(done.get(st, []))] * (NP // H) for st in (n, n + 1)}

    def cell(step, p, j):
        assert C[j % R] == j, (LO, n, step, p, j)
        k = LO + j - n - 1
        assert -NMAT <= k <= NN - 1
        rate = LO + p
        assert k == rate - step - 1
        done.setdefault(step, []).append(rate)

    c = 0
    while c * CH < NP:
        if c >= c0:
            if c == c0:
                for j in range(c * CH - 2, c * CH + P):
                    if j < NP:
                        C[j % R] = j
            for p in range(c * CH, min((c + 1) * CH, NP)):
                if p + P < NP:
                    C[(p + P) % R] = p + P
                cell(n, p, p)
                if p >= 1:
                    cell(n + 1, p - 1, p - 2)
                if p % H == H - 1:
                    caps[n][p // H] = list(done.get(n, []))
                if p >= 1 and (p - 1) % H == H - 1:
                    caps[n + 1][(p - 1) // H] = list(done.get(n + 1, []))
        c += 1
    cell(n + 1, NP - 1, NP - 2)
    caps[n + 1][NP // H - 1] = list(done.get(n + 1, []))
    return caps


@pytest.mark.parametrize("ch", [4, 8])
def test_long_tenor_forward_passes(ch):
    """k_tpq's forward in two passes of 80 rates at NN=160, NMAT=120: pass 1
    (rates 0..79) runs the step pairs n < 79, pass 2 (rates 80..159) every
    pair from pass 1's drift sums at rate 79. Every active cell runs exactly
    once, each step's cells run up the rates in order (the drift sum's
    chain), each rate's steps run in order, and the sums saved at the block
    tops (rates 39, 79, 119, 159) hold exactly the step's active cells at or
    below the top."""
    NN, NMAT, H, P = 160, 120, 40, 1
    HF = 2 * H
    done = {}
    saved = {}
    for n in range(0, NMAT, 2):
        if n < HF - 1:
            caps = fwd_pair_pass(HF, H, ch, P, 0, n, NMAT, NN, done)
        else:
            caps = {n: [[] for _ in range(HF // H)], n + 1: [[] for _ in range(HF // H)]}
        for s in (n, n + 1):
            for q in range(HF // H):
                saved[(s, q)] = [r for r in caps[s][q] if r > s]
    for n in range(0, NMAT, 2):
        caps = fwd_pair_pass(NN - HF, H, ch, P, HF, n, NMAT, NN, done)
        for s in (n, n + 1):
            for q in range(2):
                saved[(s, HF // H + q)] = [r for r in caps[s][q] if r > s]
    order_by_rate = {}
    for s in sorted(done):
        active = [r for r in done[s] if r > s]
        assert active == sorted(active) and len(set(active)) == len(active), s
        assert active == list(range(s + 1, NN)), s
        for r in active:
            order_by_rate.setdefault(r, []).append(s)
    for r, steps in order_by_rate.items():
        assert steps == sorted(steps)
    for (s, b), rates in saved.items():
        assert rates == list(range(s + 1, min(b * H + H, NN))), (s, b)


def fwd_pair_rcp2(NN, CH, n, first=1):
    """Replays fwd_pair_window_cap with LMM_FWD_RCP2 (csrc/lmm_f32_tpp.cu):
    steps n, n+1 over NN rates; returns, per cell (step, rate), the
    reciprocal pair it took its 1/(IL + delta) from, as ((rate a, version of
    a), (rate b, version of b), which), a version being the number of cells
    run on the rate before. Every cell must take the reciprocal of its own
    rate's current value."""
    ver = [0] * NN
    used = {}
    c0 = (n + 1) // CH if n + 1 > 0 else 0
    t0n = t1n = None

    def pair(a, b):
        pr = ((a, ver[a]), (b, ver[b]))
        return (pr, 0), (pr, 1)

    def cell(step, i, t):
        (pr, which) = t
        assert pr[which] == (i, ver[i]), (n, step, i, pr, which, ver[i])
        used[(step, i)] = t
        ver[i] += 1

    c = 0
    while c * CH < NN:
        if c >= c0:
            if c == c0 and c * CH >= 2:
                _, t1n = pair(c * CH - 2, c * CH - 1)
            for p in range(c * CH, min((c + 1) * CH, NN)):
                if p % 2 == 0:
                    t, t0n = pair(p, p + 1)
                else:
                    t = t0n
                if p >= first:
                    cell(n, p, t)
                if p % 2 == 1:
                    ta, t1n = pair(p - 1, p)
                    if p - 1 >= first:
                        cell(n + 1, p - 1, ta)
                elif p - 1 >= first:
                    cell(n + 1, p - 1, t1n)
        c += 1
    cell(n + 1, NN - 1, t1n)
    return used


@pytest.mark.parametrize("ch", [2, 4, 8, 16])
def test_forward_reciprocal_pairs(ch):
    """With LMM_FWD_RCP2 the fused forward's skewed step pairs and the
    forward-only kernel's single steps (fwd_step_chunked) share each MUFU
    reciprocal between the cells of one step at positions 2m and 2m+1, in
    the same argument order: every cell takes the reciprocal of its own
    rate's value at the cell, and both kernels form the same pairs, so they
    round alike (the forward/backward pair reproduces the fused value)."""
    NN = 80
    for n in range(0, 40, 2):
        used = fwd_pair_rcp2(NN, ch, n)
        for step in (n, n + 1):
            c0 = (step + 1) // ch
            for i in range(max(1, c0 * ch), NN):
                (pr, which) = used[(step, i)]
                assert pr[0][0] == i - i % 2 and pr[1][0] == i - i % 2 + 1 and which == i % 2, (step, i, pr)


@pytest.mark.parametrize("ch", [2, 4, 16])
def test_long_tenor_forward_reciprocal_pairs(ch):
    """LMM_FWD_RCP2_LONG in k_tpq's forward passes (fwd_pair_pass, every cell
    of the pass runs, from local position 0) and in the thread pair's blocks
    (tp2_fwd_pair, the same body): each cell takes the reciprocal of its own
    rate's current value, from the pair of local positions (2m, 2m+1); the
    passes and blocks start at even rates (0, 40, 80, 120), so both kernels
    pair the global rates (2m, 2m+1) alike."""
    for NP, LO in ((80, 0), (80, 80), (40, 40)):
        assert LO % 2 == 0
        for n in range(0, 120, 2):
            if n - LO >= NP - 1:
                continue
            used = fwd_pair_rcp2(NP, ch, n - LO, first=0)
            for (step, i), (pr, which) in used.items():
                assert pr[0][0] == i - i % 2 and pr[1][0] == i - i % 2 + 1 and which == i % 2
