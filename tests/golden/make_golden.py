"""Generate the golden vectors in tests/golden/ from an independent restatement.

    python tests/golden/make_golden.py

This is a second, pure-Python restatement of the reference's leaf-BVH path
(src/Neighbors/BVHTraverse.jl), written with numpy float32 scalars so every
single-precision operation rounds exactly as Julia's does.  It shares no code
with the C oracle (oracle/naiveref.c), so agreement between the two pins the
oracle.  The cases are the reference's own hand fixture (the 8 points of
test/BVHTraverse.jl:165-174) plus small seeded uniform-cube cases with the
shapes of its parametric families (test/BVHTraverse.jl:225-287).
"""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
F = np.float32
I32_MAX = 2**31 - 1

# test/BVHTraverse.jl:165-169
POSITION8 = [(0.1, 0.1, 0.1), (0.2, 0.2, 0.2), (0.346, 0.98, 0.12), (0.01, 0.76, 0.99),
             (0.1111, 0.4, 0.31), (0.234, 0.29, 0.2), (0.11346, 0.918, 0.1276),
             (0.061, 0.76, 0.989)]


def wrap32(v: int) -> int:
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= (1 << 31) else v


def jl_min(x, y):
    d = F(x - y)
    return x if np.signbit(d) else y


def jl_max(x, y):
    d = F(x - y)
    return y if np.signbit(d) else x


def morton(pos):
    """mortoncodes! (BVHTraverse.jl:241-283), Float32 / binwidth then floor."""
    bw = F(1.0 / 1023.0)
    magic = (153391689, 306783378, 613566756)
    codes = []
    for p in pos:
        c = 0
        for d in range(3):
            q = int(np.floor(F(F(p[d]) / bw)))
            yin = q & magic[d]
            yang = q | wrap32(~magic[d])
            c |= yin & yang
        codes.append(wrap32(c))
    return codes


def delta(i, code, nL, apl):
    """exptdelta (BVHTraverse.jl:677-696), 1-based leaf index."""
    if i >= nL or i < 1:
        return I32_MAX
    x = (code[(i - 1) * apl] ^ code[i * apl]) & 0xFFFFFFFF
    add = (0x80000000 + (i ^ (i + 1))) if x == 0 else 0
    return wrap32(x + add - 1)


def build(pos_sorted, code, nL, apl, h):
    """leaf boxes + bvh_interior! (BVHTraverse.jl:376-410, 704-860) in leaf order."""
    keys = {}
    for leaf in range(1, nL + 1):
        b = (leaf - 1) * apl
        mn = [F(F(pos_sorted[b][d]) - h) for d in range(3)]
        mx = [F(F(pos_sorted[b][d]) + h) for d in range(3)]
        for a in range(b, b + apl):
            for d in range(3):
                mn[d] = jl_min(mn[d], F(F(pos_sorted[a][d]) - h))
                mx[d] = jl_max(mx[d], F(F(pos_sorted[a][d]) + h))
        keys[leaf] = [mn, mx, 0, 0]
    for k in range(nL + 1, 2 * nL):
        keys[k] = [[F(0)] * 3, [F(0)] * 3, 0, 0]
    store = [0] * nL
    for i0 in range(1, nL + 1):
        i = i0
        rl = rr = i
        dl = delta(rl - 1, code, nL, apl)
        dr = delta(rr, code, nL, apl)
        bmin = list(keys[i][0])
        bmax = list(keys[i][1])
        keys[i][3] = 0 if i == nL else ((i + 1) if dr < delta(i + 1, code, nL, apl) else nL + i + 1)
        while True:
            if dr < dl:
                left = i
                split = rr
                old = store[split]
                if old == 0:
                    store[split] = rl
                rr = old
                if rr == 0:
                    break
                dr = delta(rr, code, nL, apl)
                sib = split + 1
                if sib != rr:
                    sib = nL + sib
            else:
                split = rl - 1
                old = store[split]
                if old == 0:
                    store[split] = rr
                rl = old
                if rl == 0:
                    break
                dl = delta(rl - 1, code, nL, apl)
                left = split
                if left != rl:
                    left = nL + left
                sib = left
            for d in range(3):
                bmax[d] = jl_max(keys[sib][1][d], bmax[d])
                bmin[d] = jl_min(keys[sib][0][d], bmin[d])
            q = rr if dr < dl else rl
            parent = nL + q
            if rr == nL:
                skip = 0
            else:
                r = rr + 1
                skip = r if dr < delta(r, code, nL, apl) else nL + r
            keys[parent] = [list(bmin), list(bmax), left, skip]
            i = parent
            if i == nL + 1:
                break
    return keys


def dist2(a, b):
    dx, dy, dz = F(F(a[0]) - F(b[0])), F(F(a[1]) - F(b[1])), F(F(a[2]) - F(b[2]))
    return F(F(F(dx * dx) + F(dy * dy)) + F(dz * dz))


def overlap(a, b):
    return all((a[0][d] < b[1][d]) and (a[1][d] > b[0][d]) for d in range(3))


def leaf_traverse(keys, idx, pos, nL, apl, r):
    """leafneighbor_traverse (BVHTraverse.jl:1236-1323), one thread."""
    r2 = F(F(r) * F(r))
    out = []
    for q in range(1, nL + 1):
        A = (q - 1) * apl
        for i in range(apl - 1):
            for j in range(i + 1, apl):
                d2 = dist2(pos[A + i], pos[A + j])
                if d2 < r2:
                    out.append((idx[A + i], idx[A + j], float(np.sqrt(d2))))
        t = keys[q][3]
        while t != 0:
            nd = keys[t]
            if overlap(keys[q], nd):
                if nd[2] == 0:
                    B = (t - 1) * apl
                    for i in range(apl):
                        for j in range(apl):
                            d2 = dist2(pos[A + i], pos[B + j])
                            if d2 < r2:
                                out.append((idx[A + i], idx[B + j], float(np.sqrt(d2))))
                    t = nd[3]
                else:
                    t = nd[2]
            else:
                t = nd[3]
    return out


def atom_traverse(keys, idx, pos, n, apl, r):
    """neighbor_traverse (BVHTraverse.jl:1125-1183), made runnable."""
    r2 = F(F(r) * F(r))
    out = []
    for qi in range(1, n):
        p = pos[qi - 1]
        t = (qi + apl - 1) // apl
        while t != 0:
            nd = keys[t]
            if all(nd[0][d] < F(p[d]) < nd[1][d] for d in range(3)):
                if nd[2] == 0:
                    low = (t - 1) * apl + 1
                    for e in range(1, apl + 1):
                        s = low + e - 1
                        if qi < e + low and idx[qi - 1] != idx[s - 1]:
                            d2 = dist2(p, pos[s - 1])
                            if d2 < r2:
                                out.append((idx[qi - 1], idx[s - 1], float(np.sqrt(d2))))
                    t = nd[3]
                else:
                    t = nd[2]
            else:
                t = nd[3]
    return out


def case(name, pos, r, apl, boxes):
    pos = [tuple(F(c) for c in p) for p in pos]
    n = len(pos)
    nL = n // apl
    codes = morton(pos)
    perm = sorted(range(n), key=lambda k: (codes[k], k))  # stable sortperm
    idx = [k + 1 for k in perm]
    ps = [pos[k] for k in perm]
    cs = [codes[k] for k in perm]
    h = F(F(r) / F(2)) if boxes == "leaf" else F(r)
    keys = build(ps, cs, nL, apl, h)
    keys[nL + 1][0] = [F(0)] * 3  # root overwrite, BVHTraverse.jl:856-858
    keys[nL + 1][1] = [F(1)] * 3
    if boxes == "leaf":
        pairs = leaf_traverse(keys, idx, ps, nL, apl, r)
    else:
        pairs = atom_traverse(keys, idx, ps, n, apl, r)
    kl = [[[float(v) for v in keys[k][0]], [float(v) for v in keys[k][1]], keys[k][2], keys[k][3]]
          for k in range(1, 2 * nL)]
    return dict(name=name, r=float(F(r)), apl=apl, boxes=boxes,
                position=[[float(c) for c in p] for p in pos], codes=codes,
                perm=[k + 1 for k in perm], index=idx, code_sorted=cs, keys=kl,
                pairs=[[int(a), int(b), float(d)] for (a, b, d) in pairs])


def main():
    rng = np.random.default_rng(0x4E44)
    cases = [case("position8_apl1_r10_atom", POSITION8, 10.0, 1, "atom"),
             case("position8_apl2_r0.5_leaf", POSITION8, 0.5, 2, "leaf"),
             case("position8_apl4_r0.3_leaf", POSITION8, 0.3, 4, "leaf")]
    for n, r, apl in [(64, 0.3, 4), (100, 0.1, 5), (60, 0.25, 2), (40, 0.35, 4)]:
        pos = rng.random((n, 3)).astype(np.float32)
        cases.append(case(f"uniform{n}_apl{apl}_r{r}_leaf", pos.tolist(), r, apl, "leaf"))
        cases.append(case(f"uniform{n}_apl{apl}_r{r}_atom", pos.tolist(), r, apl, "atom"))
    # duplicated points: equal Morton codes exercise the index tie-break in exptdelta
    dup = rng.random((8, 3)).astype(np.float32)
    dup = np.concatenate([dup, dup, dup[:4]]).tolist()
    cases.append(case("duplicates20_apl4_r0.5_leaf", dup, 0.5, 4, "leaf"))
    with open(os.path.join(HERE, "bvh_golden.json"), "w") as f:
        json.dump(cases, f, separators=(",", ":"))
    print(f"wrote {len(cases)} cases")


if __name__ == "__main__":
    main()
