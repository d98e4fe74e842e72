"""The early stop of the packed score and trace passes, checked on the
reference recurrence on the CPU (no GPU).

The passes sweep a pair's matrix as a wavefront: lane l of a group of G lanes
owns rows l*RPL+1 .. l*RPL+RPL and has computed columns 1 .. s-l+1 after step
s.  After step s = 16 m + G - 1 they bound every cell not computed yet by

    max(match * L_m,  H(f) + match * min(Q - i, L_m)  over the cells f = (i, j)
                      with a successor not computed yet)

with L_m = LCS(query, window columns 16 m + 1 .. R), the suffix value the LCS
pass stores.  The cells f are each row's current cell and, for a lane's last
row, the cell one column back.  The trace pass stops once the bound is below
the pair's maximum so far, the score pass once it is at most that maximum or
once bound and maximum are both below the least score that could make the pair
its group's pick.  These tests compute whole matrices of the reference
recurrence (src/smithWaterman.cu:510-645: gap_ext after a gap of the same
direction, gap_open otherwise; ties NONE > DIAG > UP > LEFT; the first maximum
in row-major order), pinned to the oracle's Smith-Waterman, and check at every
test point that

  * every cell not computed yet is at most the bound,
  * when the trace pass would stop, the first maximum is already computed and
    every cell its traceback visits too,
  * when the score pass would stop on the threshold T, the pair's score is
    below T;

and that the LCS pass's scan (the query reversed into the top bits of its
bit vector, the window from its last column down) yields exactly those suffix
values.
"""
import random

import pytest

M, X, O, E = 2, -1, -10, -1
NONE, DIAG, UP, LEFT = 0, 1, 2, 3


def reference_dp(q: bytes, w: bytes):
    """H and directions of the reference recurrence; (best, row, col) of the
    first maximum in row-major order."""
    Q, R = len(q), len(w)
    H = [[0] * (R + 1) for _ in range(Q + 1)]
    D = [[NONE] * (R + 1) for _ in range(Q + 1)]
    best, bi, bj = 0, 0, 0
    for i in range(1, Q + 1):
        for j in range(1, R + 1):
            d = H[i - 1][j - 1] + (M if q[i - 1] == w[j - 1] else X)
            u = H[i - 1][j] + (E if D[i - 1][j] == UP else O)
            l = H[i][j - 1] + (E if D[i][j - 1] == LEFT else O)
            v, dd = 0, NONE
            if v < d:
                v, dd = d, DIAG
            if v < u:
                v, dd = u, UP
            if v < l:
                v, dd = l, LEFT
            H[i][j], D[i][j] = v, dd
            if v > best:
                best, bi, bj = v, i, j
    return H, D, best, bi, bj


def traceback_cells(D, i, j):
    cells = []
    while i > 0 and j > 0:
        cells.append((i, j))
        d = D[i][j]
        if d == DIAG:
            i, j = i - 1, j - 1
        elif d == UP:
            i -= 1
        elif d == LEFT:
            j -= 1
        else:
            break
    return cells


def lcs(a: bytes, b: bytes) -> int:
    prev = [0] * (len(b) + 1)
    for x in a:
        cur = [0] * (len(b) + 1)
        for k, y in enumerate(b, 1):
            cur[k] = prev[k - 1] + 1 if x == y else max(prev[k], cur[k - 1])
        prev = cur
    return prev[-1]


def check_points(Q, R, G, RPL):
    """(m, J) per early-stop test: J[i] = the last computed column of row i."""
    steps = R + G - 1
    m = 1
    while 16 * m + G - 1 < steps:
        s = 16 * m + G - 1
        J = [0] + [min(R, s - (i - 1) // RPL + 1) for i in range(1, Q + 1)]
        yield m, J
        m += 1


def bound(H, J, Q, RPL, L):
    b = M * L
    for i in range(1, Q + 1):
        gain = M * max(0, min(Q - i, L))
        b = max(b, H[i][J[i]] + gain)
        if i % RPL == 0 and J[i] >= 2:  # a lane's last row: the cell one column back
            b = max(b, H[i][J[i] - 1] + gain)
    return b


def planted(rng, Q, R, subs, indels):
    """A query, and a window holding a mutated copy of it at a random offset."""
    q = bytes(rng.choice(b"ACGT") for _ in range(Q))
    copy = bytearray(q)
    for _ in range(subs):
        k = rng.randrange(len(copy))
        copy[k] = rng.choice([c for c in b"ACGT" if c != copy[k]])
    for _ in range(indels):
        k = rng.randrange(len(copy))
        if rng.random() < 0.5:
            del copy[k]
        else:
            copy.insert(k, rng.choice(b"ACGT"))
    w = bytearray(rng.choice(b"ACGT") for _ in range(R))
    off = rng.randrange(0, R - len(copy))
    w[off:off + len(copy)] = copy
    return q, bytes(w)


def cases(seed, n, Q, R):
    rng = random.Random(seed)
    out = []
    for k in range(n):
        kind = k % 4
        if kind == 0:
            out.append(planted(rng, Q, R, 0, 0))
        elif kind == 1:
            out.append(planted(rng, Q, R, rng.randrange(1, 4), rng.randrange(0, 2)))
        elif kind == 2:  # no true window
            out.append((bytes(rng.choice(b"ACGT") for _ in range(Q)),
                        bytes(rng.choice(b"ACGT") for _ in range(R))))
        else:  # low complexity: many equal scores
            unit = bytes(rng.choice(b"AC") for _ in range(rng.randrange(2, 5)))
            q = (unit * Q)[:Q]
            w = bytes(rng.choice(b"ACG") if rng.random() < 0.2 else c for c in (unit * R)[:R])
            out.append((q, w))
    return out


def test_reference_dp_matches_oracle(oracle):
    for q, w in cases(5, 24, 30, 90):
        _, _, best, bi, bj = reference_dp(q, w)
        a = oracle.sw(q, w, m=M, x=X, o=O, e=E)
        assert a["score"] == best
        if best > 0:
            assert a["cell_max"] == bi * (len(w) + 1) + bj


@pytest.mark.parametrize("G,RPL", [(8, 4), (4, 8), (2, 16), (16, 2)])
def test_bound_covers_the_cells_left(G, RPL):
    Q, R = 30, 140
    stops = 0
    for q, w in cases(11 + G, 64, Q, R):
        H, D, best, bi, bj = reference_dp(q, w)
        path = traceback_cells(D, bi, bj) if best > 0 else []
        for m, J in check_points(Q, R, G, RPL):
            L = lcs(q, w[16 * m:])
            b = bound(H, J, Q, RPL, L)
            left = [H[i][j] for i in range(1, Q + 1) for j in range(J[i] + 1, R + 1)]
            assert max(left, default=0) <= b
            so_far = max(H[i][j] for i in range(1, Q + 1) for j in range(1, J[i] + 1))
            if b < so_far:
                # the trace pass stops here: its first maximum and traceback are done
                stops += 1
                assert so_far == best and bj <= J[bi]
                assert all(j <= J[i] for i, j in path)
                break
    assert stops > 0  # the planted pairs stop before the window's end


def test_threshold_stop_of_the_score_pass():
    Q, R, G, RPL = 30, 140, 8, 4
    stops = 0
    pairs = cases(23, 64, Q, R)
    for t, (q, w) in enumerate(pairs):
        _, _, best_other, _, _ = reference_dp(*pairs[(t + 1) % len(pairs)])
        H, _, best, _, _ = reference_dp(q, w)
        T = best_other + (t % 2)  # a candidate's score, + 1 after it in group order
        for m, J in check_points(Q, R, G, RPL):
            L = lcs(q, w[16 * m:])
            b = bound(H, J, Q, RPL, L)
            so_far = max(H[i][j] for i in range(1, Q + 1) for j in range(1, J[i] + 1))
            if b <= so_far:
                assert so_far == best  # the score is settled
                break
            if b < T and so_far < T:
                stops += 1
                assert best < T  # reported below T, as the true score is
                break
    assert stops > 0


def suffix_lcs_by_reverse_scan(q: bytes, w: bytes, nw: int):
    """The LCS pass's scan (sw_lcs.cu): Hyyro's bit-vector LCS over 32 * nw
    bits, the query reversed into the top len(q) bits (the bits below match
    nothing), the window from its last column down; after each 16-column
    block m (columns 16 m + 1 .. R, one-based) the zeros among the query's
    bits are LCS(q, w[16 m:])."""
    T = 32 * nw
    full = (1 << T) - 1
    qmask = ((1 << len(q)) - 1) << (T - len(q))
    pm = {}
    for i, c in enumerate(q):  # query position i to bit T - 1 - i
        pm[c] = pm.get(c, 0) | (1 << (T - 1 - i))
    v = full
    out = {}
    for j in range(len(w) - 1, -1, -1):
        m_c = pm.get(w[j], 0)
        u = v & m_c
        v = ((v + u) | (v & ~m_c)) & full
        if j % 16 == 0:
            out[j // 16] = bin(~v & qmask).count("1")
    return out


def test_reverse_scan_gives_the_suffix_values():
    rng = random.Random(31)
    for q, w in cases(41, 24, 30, 100) + cases(43, 8, 100, 300):
        nw = (len(q) + 31) // 32
        got = suffix_lcs_by_reverse_scan(q, w, nw)
        assert sorted(got) == list(range((len(w) - 1) // 16 + 1))
        for m, z in got.items():
            assert z == lcs(q, w[16 * m:])
    # a query shorter than its words leaves inert bits below it
    q, w = planted(rng, 40, 120, 2, 1)
    assert suffix_lcs_by_reverse_scan(q, w, 4)[0] == lcs(q, w)
