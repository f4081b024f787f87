"""A plain-Python model of merge_up's boundary step (dmsc/src/grid_mscomplex.cpp:
24-156, cancelPairs in dmsc/include/discreteMorseAlgorithm.h:348-464) on the
complexes of two pieces, run either in the loop's row-major order or in the
ordered-parallel rounds of the device kernel (k_merge_up_rounds): each round
every pending task reserves its footprint, tasks sharing a point form one
group, and the smallest task of each group runs.  Test infrastructure for the
rounds rule; the device code is checked against the oracle by the gpu tests."""
from collections import defaultdict

CANC, STRANG, BC = 1, 2, 4


class Rect:
    def __init__(self, l, b, r, t):
        self.l, self.b, self.r, self.t = int(l), int(b), int(r), int(t)

    def contains(self, x, y):
        return self.l <= x <= self.r and self.b <= y <= self.t

    def interior(self, x, y):
        return self.l < x < self.r and self.b < y < self.t

    def boundary(self, x, y):
        return self.contains(x, y) and not self.interior(x, y)


def _lists(d, which):
    off, val = d[which + "_off"], d[which]
    out = []
    for i in range(len(off) - 1):
        c = defaultdict(int)
        for v in val[off[i]:off[i + 1]]:
            c[int(v)] += 1
        out.append(c)
    return out


def union(d1, d2, ixn):
    """merge_up's union and connectivity (:56-121) of two exported complexes."""
    cid, flags, pair, asc, des, idx = [], [], [], [], [], {}
    srcs = []
    for i, d in enumerate((d1, d2)):
        cells = [tuple(int(v) for v in c) for c in d["cellid"]]
        srcs.append((d, cells, _lists(d, "asc"), _lists(d, "des")))
        for j, c in enumerate(cells):
            if (i == 1 and c in idx) or d["flags"][j] & CANC:
                continue
            idx[c] = len(cid)
            cid.append(c)
            flags.append(int(d["flags"][j]) & (CANC | STRANG | BC))
            pair.append(None)
            asc.append(defaultdict(int))
            des.append(defaultdict(int))
    for i, (d, cells, A, D) in enumerate(srcs):
        for j, c in enumerate(cells):
            if d["flags"][j] & CANC:
                continue
            k = idx[c]
            if d["flags"][j] & BC:
                pair[k] = idx[cells[int(d["pair_idx"][j])]]
            cmn = i == 1 and ixn.contains(*c)
            for L, out in ((A[j], asc), (D[j], des)):
                for r, n in L.items():
                    cc = cells[r]
                    if (cmn and ixn.contains(*cc)) or d["flags"][r] & CANC:
                        continue
                    out[k][idx[cc]] += n
    return dict(cid=cid, flags=flags, pair=pair, asc=asc, des=des, idx=idx)


def tasks(G, rect, ext, ixn):
    """One task per boundary cell, row-major: (point, partner or None when the
    cell can never act)."""
    out = []
    for y in range(ixn.b, ixn.t + 1):
        for x in range(ixn.l, ixn.r + 1):
            si = G["idx"][(x, y)]
            pi = G["pair"][si]
            ok = pi is not None and (rect.interior(x, y) or ext.boundary(x, y)) and \
                (rect.interior(*G["cid"][pi]) or ext.boundary(*G["cid"][pi]))
            out.append((si, pi if ok else None))
    return out


def footprint(G, t):
    si, pi = t
    if pi is None or (G["flags"][si] & CANC) or not (G["flags"][si] & BC):
        return {si}
    s = {si, pi}
    for c in (si, pi):
        s |= set(G["asc"][c])
        s |= set(G["des"][c])
    return s


def run(G, t):
    """The loop body for one cell: cancelPairs of the cell's pair."""
    si, pi = t
    flags, asc, des = G["flags"], G["asc"], G["des"]
    if pi is None or (flags[si] & CANC) or not (flags[si] & BC):
        return
    c0, c1 = si, pi
    if c1 not in asc[c0]:
        c0, c1 = c1, c0
    if c1 not in asc[c0]:
        return
    for a, ca in list(asc[c0].items()):
        if a == c1:
            continue
        for d, cd in list(des[c1].items()):
            if d == c0:
                continue
            des[a][d] += ca * cd
            asc[d][a] += ca * cd
            if des[a][d] >= 2:
                flags[a] |= STRANG
                flags[d] |= STRANG
    for a in list(asc[c0]):
        if a != c1:
            des[a].pop(c0, None)
    for d in list(des[c0]):
        asc[d].pop(c0, None)
    for a in list(asc[c1]):
        des[a].pop(c1, None)
    for d in list(des[c1]):
        if d != c0:
            asc[d].pop(c1, None)
    flags[c0] |= CANC
    flags[c1] |= CANC
    des[c0].clear()
    asc[c1].clear()


def run_rounds(G, T, budget=None):
    """The rounds schedule; past `budget` pending-task evaluations the rest
    runs in order, as the kernel's finishing thread does.  Returns the rounds."""
    pending = list(range(len(T)))
    rounds = work = 0
    while pending:
        work += len(pending)
        if budget is not None and work > budget:
            for t in pending:
                run(G, T[t])
            break
        rounds += 1
        fp = {t: footprint(G, T[t]) for t in pending}
        slot = {}
        for t in pending:
            for c in fp[t]:
                slot.setdefault(c, t)
        parent = {t: t for t in pending}

        def root(a):
            while parent[a] != a:
                parent[a] = parent[parent[a]]
                a = parent[a]
            return a

        for t in pending:
            for c in fp[t]:
                ra, rb = root(t), root(slot[c])
                if ra != rb:
                    parent[max(ra, rb)] = min(ra, rb)
        commit = [t for t in pending if root(t) == t]
        for t in commit:
            run(G, T[t])
        done = set(commit)
        pending = [t for t in pending if t not in done]
    return rounds


def same(G, H):
    if G["flags"] != H["flags"]:
        return False
    for k in ("asc", "des"):
        for a, b in zip(G[k], H[k]):
            if {x: v for x, v in a.items() if v} != {x: v for x, v in b.items() if v}:
                return False
    return True


# merge_down's uncancellation along the boundary (grid_mscomplex.cpp:172-201,
# uncancel_pairs in discreteMorseAlgorithm.h:1006-1089), on the merged parent.

def down_tasks(G, rect, ext, ixn):
    """One task per boundary cell, reverse row-major."""
    out = []
    for y in range(ixn.t, ixn.b - 1, -1):
        for x in range(ixn.r, ixn.l - 1, -1):
            si = G["idx"][(x, y)]
            pi = G["pair"][si]
            ok = pi is not None and (rect.interior(x, y) or ext.boundary(x, y)) and \
                (rect.interior(*G["cid"][pi]) or ext.boundary(*G["cid"][pi]))
            out.append((si, pi if ok else None))
    return out


def down_footprint(G, t):
    si, pi = t
    if pi is None or not (G["flags"][si] & CANC):
        return {si}
    s = {si, pi}
    for c in (si, pi):
        for L in (G["asc"][c], G["des"][c]):
            for r in L:
                s.add(r)
                if G["flags"][r] & BC and G["pair"][r] is not None:
                    s.add(G["pair"][r])
    return s


def run_down(G, t):
    si, pi = t
    flags, asc, des, pair = G["flags"], G["asc"], G["des"], G["pair"]
    if pi is None or not (flags[si] & CANC):
        return
    c1, c2 = si, pi
    if c2 not in asc[c1]:
        c1, c2 = c2, c1
    for i, (L, other) in enumerate(((asc[c1], c2), (des[c2], c1))):
        assert other in L, "cancellable pair is not connected"
        new = defaultdict(int)
        for rx, cx in list(L.items()):
            if rx == other:
                continue
            if not (flags[rx] & BC):
                new[rx] += cx
                continue
            assert not (flags[rx] & CANC)
            p = pair[rx]
            for ry, cy in (asc[p] if i == 0 else des[p]).items():
                new[ry] += cx * cy
        L.clear()
        L.update(new)
    flags[c1] &= ~CANC
    flags[c2] &= ~CANC


def run_down_rounds(G, T):
    """The rounds schedule of run_rounds with the uncancellation's footprint."""
    pending, rounds = list(range(len(T))), 0
    while pending:
        rounds += 1
        fp = {t: down_footprint(G, T[t]) for t in pending}
        slot = {}
        for t in pending:
            for c in fp[t]:
                slot.setdefault(c, t)
        parent = {t: t for t in pending}

        def root(a):
            while parent[a] != a:
                parent[a] = parent[parent[a]]
                a = parent[a]
            return a

        for t in pending:
            for c in fp[t]:
                ra, rb = root(t), root(slot[c])
                if ra != rb:
                    parent[max(ra, rb)] = min(ra, rb)
        commit = [t for t in pending if root(t) == t]
        for t in commit:
            run_down(G, T[t])
        done = set(commit)
        pending = [t for t in pending if t not in done]
    return rounds
