"""Pure-Python restatement of the symbolic analysis (small cases only).

TEST INFRASTRUCTURE ONLY (the checker for the library's host compiler).

The reference (CedarSim) leaves structure to DAECompiler and solves densely; the
sparse structure below is the documented algorithm of this project, restated
independently so that the library's J pattern, static pivot (row matching),
fill-reducing order and LU fill can be compared bit for bit:

  * structural J pattern: from each device's equations (which KCL / branch rows
    depend on which unknowns), src/simpledevices.jl and the VA contribution rules
    of src/vasim.jl:128-180;
  * matching: diagonal first; then for each unmatched column in increasing order a
    free row of that column (increasing row order), else a depth-first augmenting
    path visiting rows in increasing order (Duff 1981);
  * ordering: exact minimum degree on B + B^T (B = row-matched J), ties -> lowest
    index; node diagonals join the pattern after matching;
  * LU fill: symbolic Gaussian elimination without pivoting in that order.
"""
from __future__ import annotations

from typing import Dict, List, Set, Tuple

R, C, L, V, I, E, G, MOS1, DIODE, NLVCR = range(1, 11)


def device_structure(model: int, t: List[int]) -> Set[Tuple[int, int]]:
    """(row, col) pairs a device makes structurally nonzero (ground = -1 dropped)."""
    pairs: Set[Tuple[int, int]] = set()

    def add(rows, cols):
        for r in rows:
            for c in cols:
                if r >= 0 and c >= 0:
                    pairs.add((r, c))

    if model in (R, C, DIODE):          # current/charge depends on V(p,n), enters KCL p, n
        add(t[0:2], t[0:2])
    elif model == L:                     # KCL p,n <- I ; branch row <- V(p,n), I
        add(t[0:2], [t[2]]); add([t[2]], [t[0], t[1], t[2]])
    elif model == V:                     # KCL p,n <- I ; branch row <- V(p,n)
        add(t[0:2], [t[2]]); add([t[2]], t[0:2])
    elif model == I:
        pass
    elif model == E:                     # KCL p,n <- I ; branch row <- V(p,n), V(cp,cn)
        add(t[0:2], [t[4]]); add([t[4]], t[0:4])
    elif model == G:                     # KCL p,n <- V(cp,cn)
        add(t[0:2], t[2:4])
    elif model in (MOS1, NLVCR):         # I(d,s) depends on d, g, s; enters KCL d, s
        add([t[0], t[2]], t[0:3])
    return pairs


def structure(flat) -> Set[Tuple[int, int]]:
    from itertools import chain
    pat: Set[Tuple[int, int]] = set()
    for (model, term, br, par) in flat.groups:
        for i in range(term.shape[0]):
            tt = [int(v) for v in term[i]]
            if br is not None:
                tt.append(int(br[i]))
            pat |= device_structure(model, tt)
    return pat


def csc(pat: Set[Tuple[int, int]], n: int):
    cols: Dict[int, List[int]] = {c: [] for c in range(n)}
    for (r, c) in pat:
        cols[c].append(r)
    colptr, rowidx = [0], []
    for c in range(n):
        rowidx += sorted(cols[c])
        colptr.append(len(rowidx))
    return colptr, rowidx


def matching(pat: Set[Tuple[int, int]], n: int) -> List[int]:
    colrows = [sorted(r for (r, c) in pat if c == u) for u in range(n)]
    mrow = [-1] * n
    mcol = [-1] * n
    for u in range(n):
        if (u, u) in pat:
            mrow[u] = u; mcol[u] = u
    for u0 in range(n):
        if mcol[u0] >= 0:
            continue
        free = [e for e in colrows[u0] if mrow[e] < 0]
        if free:
            mrow[free[0]] = u0; mcol[u0] = free[0]
            continue
        visited = set()

        def dfs(u):
            for e in colrows[u]:
                if e in visited:
                    continue
                visited.add(e)
                if mrow[e] < 0 or dfs(mrow[e]):
                    mrow[e] = u; mcol[u] = e
                    return True
            return False

        if not dfs(u0):
            raise ValueError("structurally singular")
    return mcol


def min_degree(adj: List[Set[int]]) -> List[int]:
    adj = [set(a) for a in adj]
    alive = set(range(len(adj)))
    order = []
    while alive:
        v = min(alive, key=lambda k: (len(adj[k]), k))
        order.append(v)
        alive.remove(v)
        nb = list(adj[v])
        for a in nb:
            adj[a].discard(v)
            adj[a] |= (set(nb) - {a})
        adj[v] = set()
    return order


def analyze(flat):
    """Return (colptr, rowidx, rowmatch, order, lu_colptr, lu_rowidx)."""
    n = flat.n
    pat = structure(flat)
    colptr, rowidx = csc(pat, n)
    rm = matching(pat, n)
    eq2u = {rm[u]: u for u in range(n)}
    adj = [set() for _ in range(n)]
    pat2 = set(pat) | {(u, u) for u in range(flat.n_nodes)}
    for (e, u) in pat2:
        up = eq2u[e]
        if up != u:
            adj[up].add(u); adj[u].add(up)
    order = min_degree(adj)
    iorder = {u: p for p, u in enumerate(order)}
    eqpos = {rm[u]: iorder[u] for u in range(n)}
    rows = [set() for _ in range(n)]
    for (e, u) in pat2:
        rows[eqpos[e]].add(iorder[u])
    for k in range(n):
        upper = {q for q in rows[k] if q > k}
        for i in range(k + 1, n):
            if k in rows[i]:
                rows[i] |= upper
    lu = {(p, q) for p in range(n) for q in rows[p]}
    lcp, lri = csc(lu, n)
    return colptr, rowidx, rm, order, lcp, lri


def nested_dissection(adj: List[Set[int]]) -> List[int]:
    """Level-structure nested dissection (George 1973): dense vertices last; split
    each component at the middle BFS level from a pseudo-peripheral vertex."""
    import math
    n = len(adj)
    thresh = max(16, int(4.0 * math.sqrt(n)))
    dense = [len(adj[v]) > thresh for v in range(n)]
    order: List[int] = []

    def bfs(root, member):
        levels, cur, seen = [], [root], {root}
        while cur:
            cur = sorted(cur)
            levels.append(cur)
            nxt = []
            for v in cur:
                for w in sorted(adj[v]):
                    if w in member and w not in seen:
                        seen.add(w); nxt.append(w)
            cur = nxt
        return levels

    def nd(V):
        V = sorted(V)
        member = set(V)
        comps, seen = [], set()
        for v in V:
            if v in seen:
                continue
            comp, k = [v], 0
            seen.add(v)
            while k < len(comp):
                for w in sorted(adj[comp[k]]):
                    if w in member and w not in seen:
                        seen.add(w); comp.append(w)
                k += 1
            comps.append(sorted(comp))
        if len(comps) > 1:
            for c in comps:
                nd(c)
            return
        C = comps[0]
        if len(C) <= 3:
            order.extend(C)
            return
        member = set(C)
        deg = lambda v: sum(1 for w in adj[v] if w in member)
        levels = bfs(C[0], member)
        for _ in range(5):
            u = min(levels[-1], key=lambda v: (deg(v), v))
            lv2 = bfs(u, member)
            if len(lv2) > len(levels):
                levels = lv2
            else:
                break
        m = len(levels) - 1
        if m < 2:
            order.extend(C)
            return
        S = levels[m // 2]
        nd([v for v in C if v not in set(S)])
        order.extend(S)

    V = [v for v in range(n) if not dense[v]]
    D = [v for v in range(n) if dense[v]]
    if V:
        nd(V)
    order.extend(sorted(D, key=lambda v: len(adj[v])))
    return order


def analyze_with(flat, ordering: int):
    """analyze() with a forced ordering: 1 minimum degree, 2 nested dissection."""
    global min_degree
    if ordering == 2:
        saved = min_degree
        try:
            min_degree = nested_dissection
            return analyze(flat)
        finally:
            min_degree = saved
    return analyze(flat)
