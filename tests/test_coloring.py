"""The multicolour orderings are valid Gauss-Seidel orderings: blocks of one
colour (lines along d coloured by the parity of their transverse node
indices; node patches by the parity of (i,j,k)) write disjoint unknowns and
never read an unknown another block of the same colour writes.  Checked by
enumerating every block's write set and the read set of its rows'
finite-integration equations on small non-cubic grids."""
import itertools

import pytest


def nbrs(c, P):
    """Edges read by the equation of edge (c, P) (src/gmg.c:1365-1404)."""
    p, q = (c + 1) % 3, (c + 2) % 3
    out = []
    for dc, dp, dq, comp in [(0, 1, 0, c), (0, -1, 0, c), (0, 0, 1, c), (0, 0, -1, c),
                             (1, 0, 0, p), (0, 0, 0, p), (1, -1, 0, p), (0, -1, 0, p),
                             (1, 0, 0, q), (0, 0, 0, q), (1, 0, -1, q), (0, 0, -1, q)]:
        Q = list(P)
        Q[c] += dc
        Q[p] += dp
        Q[q] += dq
        out.append((comp, tuple(Q)))
    return out + [(c, tuple(P))]


def is_unknown(n, c, P):
    p, q = (c + 1) % 3, (c + 2) % 3
    return 0 <= P[c] < n[c] and 1 <= P[p] < n[p] and 1 <= P[q] < n[q]


def line_unknowns(n, d, ta, tb):
    a, b = (1, 2) if d == 0 else ((0, 2) if d == 1 else (0, 1))
    u = []
    for s in range(n[d]):
        P = [0, 0, 0]
        P[d], P[a], P[b] = s, ta, tb
        u.append((d, tuple(P)))
    for s in range(1, n[d]):
        for comp, da, db in [(a, -1, 0), (a, 0, 0), (b, 0, -1), (b, 0, 0)]:
            P = [0, 0, 0]
            P[d], P[a], P[b] = s, ta + da, tb + db
            u.append((comp, tuple(P)))
    return [x for x in u if is_unknown(n, *x)]


def patch_unknowns(n, N):
    u = []
    for c in range(3):
        for side in (0, 1):
            P = list(N)
            P[c] -= 1 - side
            u.append((c, tuple(P)))
    return u


def check_colour(n, blocks):
    writes = [set(b) for b in blocks]
    reads = [set(e for x in b for e in nbrs(*x) if is_unknown(n, *e)) for b in blocks]
    owner = {}
    for i, w in enumerate(writes):
        for e in w:
            assert e not in owner, f"blocks {owner[e]} and {i} both write {e}"
            owner[e] = i
    for i, r in enumerate(reads):
        for e in r:
            j = owner.get(e)
            assert j is None or j == i, f"block {i} reads {e} written by block {j}"


@pytest.mark.parametrize("n", [(6, 5, 7), (8, 8, 4), (5, 9, 6)])
@pytest.mark.parametrize("d", [0, 1, 2])
def test_line_colours_independent(n, d):
    a, b = (1, 2) if d == 0 else ((0, 2) if d == 1 else (0, 1))
    for pa, pb in itertools.product((0, 1), (0, 1)):
        blocks = [line_unknowns(n, d, ta, tb)
                  for ta in range(1, n[a]) for tb in range(1, n[b])
                  if ta % 2 == pa and tb % 2 == pb]
        check_colour(n, blocks)


@pytest.mark.parametrize("n", [(6, 5, 7), (8, 8, 4)])
def test_patch_colours_independent(n):
    for col in range(8):
        blocks = [patch_unknowns(n, (i, j, k))
                  for i in range(1, n[0]) for j in range(1, n[1]) for k in range(1, n[2])
                  if (i % 2, j % 2, k % 2) == (col & 1, (col >> 1) & 1, (col >> 2) & 1)]
        check_colour(n, blocks)


def test_lines_cover_every_unknown_once_per_direction_pair():
    """Each line direction's colours together update every E_d unknown once
    and every transverse unknown exactly twice (shared by neighbouring
    lines), as the reference's overlapping line blocks do."""
    n = (6, 5, 7)
    for d in range(3):
        a, b = (1, 2) if d == 0 else ((0, 2) if d == 1 else (0, 1))
        count = {}
        for ta in range(1, n[a]):
            for tb in range(1, n[b]):
                for e in line_unknowns(n, d, ta, tb):
                    count[e] = count.get(e, 0) + 1
        for (c, P), k in count.items():
            if c == d:
                assert k == 1
            else:
                t = a if c == a else b
                assert k == (2 if 1 <= P[t] < n[t] - 1 else 1)
