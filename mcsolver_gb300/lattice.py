"""Model builder: the MCMainFunction argument tuples of periodic lattices.

``lattice_args`` produces, for a periodic supercell of a lattice with
``norb`` orbitals per cell and a list of bonds, exactly the positional tuple
that mcsolver's ``mcMain.MC`` builds and passes to the compiled library
(site id order x, y, z, orbital as Lattice.py:172-184; links in the order of
Lattice.addLinking, merging duplicate targets as Lattice.py:34-57; the
renormalised cluster and link lists of Lattice.py:185-205 and :263-271;
J, D and h divided by T as mcMain.py:21-31, :121, :244).  It lets callers
drive the engine without mcsolver's Python object graph, and it is checked
against tuples captured from the reference's own code in the test suite.
"""
from __future__ import annotations

import numpy as np


def _lattice_links(L, norb, bonds):
    """Links per site in the reference's insertion order (Lattice.py:247-271)."""
    Lx, Ly, Lz = L
    N = Lx * Ly * Lz * norb

    def sid(x, y, z, o):
        return ((x % Lx) * Ly * Lz + (y % Ly) * Lz + (z % Lz)) * norb + o

    links = [[] for _ in range(N)]   # (target, strength)
    rlinks = [[] for _ in range(N)]
    chosen = [False] * N
    for x in range(Lx):
        for y in range(Ly):
            for z in range(Lz):
                for o in range(norb):
                    if x % 2 + y % 2 + z % 2 == 0:
                        chosen[sid(x, y, z, o)] = True

    # every link carries a tag (bond index, 0 forward / 1 inverse) of the bond
    # whose strength it holds; a second bond to the same target (duplicate
    # targets on supercells of side <= 2) is merged or dropped by comparing
    # strengths, which depends on their values, and is counted in `merged`
    merged = [0]

    def add(lst, i, j, s, merge, tag):
        for k, (t, s0, _) in enumerate(lst[i]):
            if t == j:
                if merge:
                    merged[0] += 1
                    if np.sum(np.abs(np.asarray(s0) - np.asarray(s))) < 1e-5:
                        return
                    lst[i][k] = (t, np.asarray(s0) + np.asarray(s), None)
                return
        lst[i].append((j, np.asarray(s), tag))

    for x in range(Lx):
        for y in range(Ly):
            for z in range(Lz):
                for o in range(norb):
                    i = sid(x, y, z, o)
                    for b, (src, tgt, ov, J, Jinv) in enumerate(bonds):
                        if o != src:
                            continue
                        j = sid(x + ov[0], y + ov[1], z + ov[2], tgt)
                        add(links, i, j, J, True, (b, 0))
                        if i != j:
                            add(links, j, i, Jinv, True, (b, 1))
                    if chosen[i]:
                        for b, (src, tgt, ov, J, Jinv) in enumerate(bonds):
                            if o != src:
                                continue
                            j = sid(x + 2 * ov[0], y + 2 * ov[1], z + 2 * ov[2], tgt)
                            add(rlinks, i, j, J, False, (b, 0))
                            if i != j:
                                add(rlinks, j, i, Jinv, False, (b, 1))
    return N, links, rlinks, chosen, sid, merged[0]


def lattice_args(model, L, norb, bonds, T, h=0.0, S=None, D=None, nthermal=10, nsweep=10, tau=0, algo=0,
                 ki=((0, 0), (0, 0, 0)), groups=(), circuits=(), frames=0, flunc=0.0, group_in_sc=True):
    """MCMainFunction tuple for a periodic lattice; J, D and h are divided by T
    as mcMain.py does (mcMain.py:21-31, :121, :244).  An orbital group holds
    its orbitals in every cell (group_in_sc) or in cell (0,0,0) only
    (Lattice.py:208-211)."""
    return _lattice_build(model, L, norb, bonds, T, h, S, D, nthermal, nsweep, tau, algo, ki, groups, circuits,
                          frames, flunc, group_in_sc)[0]


def _lattice_build(model, L, norb, bonds, T, h, S, D, nthermal, nsweep, tau, algo, ki, groups, circuits, frames,
                   flunc, group_in_sc):
    """lattice_args, also returning the link lists (with their bond tags) and
    the number of duplicate-target merges."""
    T = max(T, 0.1)
    S = S or [1.0] * norb
    D = D or [[0.0, 0.0, 0.0]] * norb
    on = model != "ising"
    bl = []
    for (src, tgt, ov, J9) in bonds:
        J9 = np.asarray(J9, dtype=float) / T
        if on:
            Jxx, Jyy, Jzz, Jxy, Jxz, Jyz, Jyx, Jzx, Jzy = J9
            inv = np.array([Jxx, Jyy, Jzz, Jyx, Jzx, Jzy, Jxy, Jxz, Jyz])
            bl.append((src, tgt, ov, J9, inv))
        else:
            bl.append((src, tgt, ov, J9[0], J9[0]))
    N, links, rlinks, chosen, sid, merged = _lattice_links(L, norb, bl)
    Lx, Ly, Lz = L
    z = max(len(l) for l in links)
    init = [S[i % norb] for i in range(N)]
    nlink = [len(l) for l in links]
    lo, ls = [], []
    for i in range(N):
        for k in range(z):
            if k < len(links[i]):
                lo.append(links[i][k][0])
                s = links[i][k][1]
                ls += (list(map(float, s)) if on else [float(s)])
            else:
                lo.append(-1)
                ls += ([0.0] * 9 if on else [0.0])
    rorb, rcl, rlk = [], [], []
    for x in range(Lx):
        for y in range(Ly):
            for zz in range(Lz):
                for o in range(norb):
                    i = sid(x, y, zz, o)
                    if not chosen[i]:
                        continue
                    rorb.append(i)
                    cl = []
                    for (dx, dy, dz) in ((0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0), (0, 1, 1), (1, 0, 1), (1, 1, 0), (1, 1, 1)):
                        c = sid(x + dx, y + dy, zz + dz, o)
                        if c not in cl:
                            cl.append(c)
                    rcl.append(cl)
                    rlk += [rlinks[i][k][0] if k < len(rlinks[i]) else -1 for k in range(z)]
    ncl = len(rcl[0])
    rcl = [c for cl in rcl for c in cl[:ncl]]
    cp = []
    (ks, kt), kov = ki
    for x in range(Lx):
        for y in range(Ly):
            for zz in range(Lz):
                cp += [sid(x, y, zz, ks), sid(x + kov[0], y + kov[1], zz + kov[2], kt)]
    tau = N if tau <= 0 else tau
    if not on:
        return (algo, tuple(init), nthermal, nsweep, tau, z, tuple(nlink), tuple(ls), tuple(lo), tuple(cp),
                h / T, tuple(rorb), tuple(rcl), tuple(rlk), frames), links, merged
    initD = []
    for i in range(N):
        initD += [float(d) / T for d in D[i % norb]]
    circ = []
    for x in range(Lx):
        for y in range(Ly):
            for zz in range(Lz):
                for c in circuits:
                    for (o, ov) in c:
                        circ.append(sid(x + ov[0], y + ov[1], zz + ov[2], o))
    grp = []
    maxg = 1
    if group_in_sc:
        gl = [[sid(x, y, zz, o) for o in g for x in range(Lx) for y in range(Ly) for zz in range(Lz)] for g in groups]
    else:
        gl = [[sid(0, 0, 0, o) for o in g] for g in groups]
    if gl:
        maxg = max(len(g) for g in gl)
        for g in gl:
            grp += g + [-1] * (maxg - len(g))
    ign = 1
    for i in range(N):
        for k in range(len(links[i])):
            if any(abs(v) > 1e-6 for v in links[i][k][1][3:]):
                ign = 0
    return (algo, tuple(init), tuple(initD), nthermal, nsweep, tau, z, tuple(nlink), tuple(ls), tuple(lo),
            tuple(circ), tuple(cp), len(groups), maxg, tuple(grp), flunc, h / T, tuple(rorb), tuple(rcl),
            tuple(rlk), frames, ign), links, merged


_RCL_OFFSETS = ((0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0), (0, 1, 1), (1, 0, 1), (1, 1, 0), (1, 1, 1))


def _structure_np(model, L, norb, bonds, S, D, nthermal, nsweep, tau, algo, ki, groups, circuits, frames, flunc,
                  group_in_sc):
    """The T-independent part of _lattice_build with numpy, for supercells in
    which no site holds two links (or two renormalised links) to one target.
    Returns (tuple at T = 1 with the T-dependent entries left as None, link
    bond index [N, z] (-1 = padding), link direction [N, z] (1 = reverse))
    or None when a duplicate target makes the reference's order depend on
    values.  The insertion order of Lattice.py:247-271 is a sort: the sites
    are visited in id order and, per site, the bonds in list order, each
    adding the forward link to its source and then the reverse link to its
    target; so a site's links are ordered by (visited site, bond, direction)."""
    Lx, Ly, Lz = L
    N = Lx * Ly * Lz * norb
    on = model != "ising"
    cell = np.arange(Lx * Ly * Lz, dtype=np.int64)
    cx, cy, cz = cell // (Ly * Lz), (cell // Lz) % Ly, cell % Lz

    def sid(x, y, z, o):
        return ((x % Lx) * Ly * Lz + (y % Ly) * Lz + (z % Lz)) * norb + o

    def ordered(owner_sites, step):
        own, tgt, src_site, bidx, rev = [], [], [], [], []
        for b, (src, t, ov, _) in enumerate(bonds):
            sel = owner_sites[src]
            i = sid(cx[sel], cy[sel], cz[sel], src)
            j = sid(cx[sel] + step * ov[0], cy[sel] + step * ov[1], cz[sel] + step * ov[2], t)
            m = i != j
            own += [i, j[m]]
            tgt += [j, i[m]]
            src_site += [i, i[m]]
            bidx += [np.full(len(i), b), np.full(int(m.sum()), b)]
            rev += [np.zeros(len(i), np.int64), np.ones(int(m.sum()), np.int64)]
        if not own:
            e = np.zeros(0, np.int64)
            return e, e, e, e, e
        own, tgt, src_site, bidx, rev = (np.concatenate(v).astype(np.int64) for v in (own, tgt, src_site, bidx, rev))
        order = np.lexsort((rev, bidx, src_site, own))
        own, tgt, bidx, rev = own[order], tgt[order], bidx[order], rev[order]
        counts = np.bincount(own, minlength=N)
        slot = np.arange(len(own)) - (np.cumsum(counts) - counts)[own]
        return own, tgt, bidx, rev, slot

    every = {o: np.ones(len(cell), bool) for o in range(norb)}
    own, tgt, bidx, rev, slot = ordered(every, 1)
    if len(np.unique(own * N + tgt)) != len(own):
        return None
    nlink = np.bincount(own, minlength=N)
    z = int(nlink.max()) if N else 0
    lo = np.full((N, z), -1, np.int64)
    tagb = np.full((N, z), -1, np.int64)
    tagi = np.zeros((N, z), np.int64)
    lo[own, slot], tagb[own, slot], tagi[own, slot] = tgt, bidx, rev
    # renormalised links of the chosen sites (even x, y, z), Lattice.py:185-205, :263-271
    chosen_cell = (cx % 2 == 0) & (cy % 2 == 0) & (cz % 2 == 0)
    rown, rtgt, _, _, rslot = ordered({o: chosen_cell for o in range(norb)}, 2)
    if len(np.unique(rown * N + rtgt)) != len(rown):
        return None
    rl = np.full((N, max(z, 1)), -1, np.int64)
    keep = rslot < z
    rl[rown[keep], rslot[keep]] = rtgt[keep]
    ch_cells = np.nonzero(chosen_cell)[0]
    rorb = (ch_cells[:, None] * norb + np.arange(norb)[None, :]).reshape(-1)
    rlk = rl[rorb, :z].reshape(-1)
    x, y, zc = cx[rorb // norb], cy[rorb // norb], cz[rorb // norb]
    o = rorb % norb
    cand = np.stack([sid(x + dx, y + dy, zc + dz, o) for (dx, dy, dz) in _RCL_OFFSETS], axis=1)
    dup = np.zeros(cand.shape, bool)
    for k in range(1, cand.shape[1]):
        dup[:, k] = (cand[:, :k] == cand[:, k:k + 1]).any(axis=1)
    kept = (~dup).sum(axis=1)
    ncl = int(kept[0]) if len(kept) else 0
    if len(kept) == 0 or kept.min() < ncl:
        return None
    idx = np.argsort(dup, axis=1, kind="stable")[:, :ncl]
    rcl = np.take_along_axis(cand, idx, axis=1).reshape(-1)
    (ks, kt), kov = ki
    cp = np.stack([sid(cx, cy, cz, ks), sid(cx + kov[0], cy + kov[1], cz + kov[2], kt)], axis=1).reshape(-1)
    S = S or [1.0] * norb
    init = np.asarray(S)[np.arange(N) % norb]
    tau = N if tau <= 0 else tau
    if not on:
        base = (algo, init, nthermal, nsweep, tau, z, nlink, None, lo.reshape(-1), cp, None, rorb, rcl, rlk, frames)
        return base, tagb, tagi
    circ = [sid(cx + ov[0], cy + ov[1], cz + ov[2], oo) for c in circuits for (oo, ov) in c]
    circ = np.stack(circ, axis=1).reshape(-1) if circ else np.zeros(0, np.int64)
    if group_in_sc:
        gl = [np.concatenate([sid(cx, cy, cz, oo) for oo in g]) if len(g) else np.zeros(0, np.int64) for g in groups]
    else:
        gl = [np.asarray([sid(0, 0, 0, oo) for oo in g], np.int64) for g in groups]
    maxg = 1
    grp = np.zeros(0, np.int64)
    if gl:
        maxg = max(len(g) for g in gl)
        grp = np.concatenate([np.concatenate([g, np.full(maxg - len(g), -1, np.int64)]) for g in gl])
    base = (algo, init, None, nthermal, nsweep, tau, z, nlink, None, lo.reshape(-1), circ, cp, len(groups), maxg,
            grp, flunc, None, rorb, rcl, rlk, frames, None)
    return base, tagb, tagi


# tuple positions of the arrays (for arrays=True) and of the T-dependent entries
_ISING_ARRAYS = (1, 6, 7, 8, 9, 11, 12, 13)
_ON_ARRAYS = (1, 2, 7, 8, 9, 10, 11, 14, 17, 18, 19)
_INV_PERM = [0, 1, 2, 6, 7, 8, 3, 4, 5]   # xx,yy,zz,xy,xz,yz,yx,zx,zy of the transpose (Lattice.py:137)


class LatticeTemplate:
    """The MCMainFunction tuples of one lattice at many (T, H) points.

    The structure (links in the reference's order, renormalised lists,
    correlated pairs, circuits, groups) is built once.  Each point recomputes
    only what depends on T and H: every link's coupling J/T (the J of the bond
    the link comes from, or its transpose for the reverse link), the
    anisotropy D/T, the field h/T and the off-diagonal flag.  ``at(T, h)``
    equals ``lattice_args(..., T, h=h, ...)`` value for value.  On supercells
    where two bonds of a site reach the same target (a side of 1 or 2), the
    reference merges or drops the second by comparing J/T values
    (Lattice.py:34-57), a decision that can depend on T; there every point is
    built by lattice_args.
    """

    def __init__(self, model, L, norb, bonds, S=None, D=None, nthermal=10, nsweep=10, tau=0, algo=0,
                 ki=((0, 0), (0, 0, 0)), groups=(), circuits=(), frames=0, flunc=0.0, group_in_sc=True):
        self.model, self.on = model, model != "ising"
        self.kw = dict(L=L, norb=norb, bonds=bonds, S=S, D=D, nthermal=nthermal, nsweep=nsweep, tau=tau, algo=algo,
                       ki=ki, groups=groups, circuits=circuits, frames=frames, flunc=flunc, group_in_sc=group_in_sc)
        fast = _structure_np(model, L, norb, bonds, S, D, nthermal, nsweep, tau, algo, ki, groups, circuits, frames,
                             flunc, group_in_sc)
        if fast is not None:
            self.base, self.tagb, self.tagi = fast
            self.merged = 0
        else:
            self.base, links, self.merged = _lattice_build(model, L, norb, bonds, 1.0, 0.0, S, D, nthermal, nsweep,
                                                           tau, algo, ki, groups, circuits, frames, flunc, group_in_sc)
            z = max(len(l) for l in links)
            self.tagb = np.full((len(links), z), -1, dtype=np.int64)
            self.tagi = np.zeros((len(links), z), dtype=np.int64)
            for i, l in enumerate(links):
                for k, (_, _, tag) in enumerate(l):
                    if tag is not None:
                        self.tagb[i, k], self.tagi[i, k] = tag
        self.vectorised = fast is not None
        N = self.tagb.shape[0]
        self.pad = self.tagb < 0
        self.J = np.asarray([b[3] for b in bonds], dtype=float).reshape(len(bonds), 9)
        Dn = np.asarray(D or [[0.0, 0.0, 0.0]] * norb, dtype=float)
        self.Dsite = Dn[np.arange(N) % norb]
        self.arrays = {k: np.asarray(self.base[k]) for k in (_ON_ARRAYS if self.on else _ISING_ARRAYS)
                       if self.base[k] is not None}

    def at(self, T, h=0.0, arrays=False):
        """The tuple at (T, h); with arrays=True its arrays are numpy arrays
        (what mcsolver_gb300.Problem takes without a copy into a tuple)."""
        if self.merged:
            return lattice_args(self.model, T=T, h=h, **self.kw)
        T = max(T, 0.1)
        J = self.J / T
        b = np.where(self.pad, 0, self.tagb)
        a = list(self.base)
        if self.on:
            both = np.stack([J, J[:, _INV_PERM]])               # [fwd/inv, bond, 9]
            ls = np.where(self.pad[..., None], 0.0, both[self.tagi, b])
            ign = 0 if np.any(np.abs(ls[..., 3:]) > 1e-6) else 1
            a[2] = (self.Dsite / T).reshape(-1)
            a[8] = ls.reshape(-1)
            a[16] = h / T
            a[21] = ign
            keys = _ON_ARRAYS
        else:
            ls = np.where(self.pad, 0.0, J[:, 0][b])
            a[7] = ls.reshape(-1)
            a[10] = h / T
            keys = _ISING_ARRAYS
        for k in keys:
            if k not in ((2, 8) if self.on else (7,)):
                a[k] = self.arrays[k]
            if not arrays:
                a[k] = tuple(np.asarray(a[k]).tolist())
        return tuple(a)


def J9(xx, yy=0, zz=0, xy=0, xz=0, yz=0, yx=0, zx=0, zy=0):
    return [xx, yy, zz, xy, xz, yz, yx, zx, zy]


SQ_CIRCUITS = [((0, (0, 0, 0)), (0, (1, 0, 0)), (0, (1, 1, 0))), ((0, (0, 0, 0)), (0, (1, 1, 0)), (0, (0, 1, 0)))]


def square_args(model, L, T, J=-1.0, h=0.0, dmi=0.0, D=None, nthermal=10, nsweep=10, tau=0, algo=0, frames=0,
                groups=((0,),), circuits=True):
    if model == "ising":
        bonds = [(0, 0, (1, 0, 0), J9(J)), (0, 0, (0, 1, 0), J9(J))]
        return lattice_args("ising", (L, L, 1), 1, bonds, T, h=h, nthermal=nthermal, nsweep=nsweep, tau=tau,
                            algo=algo, frames=frames)
    bonds = [(0, 0, (1, 0, 0), J9(J, J, J, xz=dmi, zx=-dmi)), (0, 0, (0, 1, 0), J9(J, J, J, yz=dmi, zy=-dmi))]
    return lattice_args(model, (L, L, 1), 1, bonds, T, h=h, D=[D or [0, 0, 0]], nthermal=nthermal, nsweep=nsweep,
                        tau=tau, algo=algo, frames=frames, groups=groups,
                        circuits=SQ_CIRCUITS if (circuits and model == "heisenberg") else ())


HC_POS = [[0.333333333, 0.666666667, 0.0], [0.666666667, 0.333333333, 0.0]]


def honeycomb_args(model, L, T, nthermal=10, nsweep=10, tau=0, algo=0, h=0.0):
    """Honeycomb, 1NN Kitaev-type J=diag(-1.5,-1.5,-1.8) with Jxy=Jyx=0.3, 2NN -0.3, Az=-0.5."""
    b1 = [(0, 1, o, J9(-1.5, -1.5, -1.8, xy=0.3, yx=0.3)) for o in ((0, 0, 0), (-1, 0, 0), (0, 1, 0))]
    b2 = [(a, a, o, J9(-0.3, -0.3, -0.3)) for a in (0, 1) for o in ((1, 0, 0), (1, 1, 0), (0, 1, 0))]
    if model == "ising":
        return lattice_args("ising", (L, L, 1), 2, [(s, t, o, J9(-1)) for (s, t, o, _) in b1], T, h=h,
                            nthermal=nthermal, nsweep=nsweep, tau=tau, algo=algo)
    return lattice_args(model, (L, L, 1), 2, b1 + b2, T, D=[[0, 0, -0.5], [0, 0, -0.5]], h=h,
                        nthermal=nthermal, nsweep=nsweep, tau=tau, algo=algo, groups=((0,), (1,)))




def rescale_args(model, args, T, T0=1.0, h=None):
    """The tuple of the same lattice at temperature T from one built at T0:
    couplings, anisotropy and field scale as 1/T (mcMain.py:21-31).  numpy
    array entries stay arrays.  h, when given, replaces the field (physical)."""
    T = max(T, 0.1)
    f = T0 / T
    a = list(args)
    if isinstance(a[1], np.ndarray):
        if model == "ising":
            a[7] = a[7] * f
            a[10] = a[10] * f if h is None else h / T
        else:
            a[2] = a[2] * f
            a[8] = a[8] * f
            a[16] = a[16] * f if h is None else h / T
        return tuple(a)
    if model == "ising":
        a[7] = tuple((np.asarray(a[7], dtype=float) * f).tolist())
        a[10] = a[10] * f
    else:
        a[2] = tuple((np.asarray(a[2], dtype=float) * f).tolist())
        a[8] = tuple((np.asarray(a[8], dtype=float) * f).tolist())
        a[16] = a[16] * f if h is None else h / T
    if model == "ising" and h is not None:
        a[10] = h / T
    return tuple(a)


def _square_link_order(Lx, Ly, step):
    """Targets and directions of the links of every site of a periodic square
    lattice (one orbital, bonds along [1 0 0] and [0 1 0]) in the order
    Lattice.establishLinking appends them (Lattice.py:247-271): as the target
    of the bonds from (x-step, y) and (x, y-step) when those sources are
    visited before the site itself, then its own two bonds, then the targets
    from sources visited later.  Returns (targets[N,4], fwd[N,4]) where fwd is
    True for a link the site owns (strength J) and False for an inverse one."""
    x = np.repeat(np.arange(Lx), Ly)
    y = np.tile(np.arange(Ly), Lx)
    sid = lambda a, b: (a % Lx) * Ly + (b % Ly)
    tA = sid(x - step, y)          # inverse of bond 0 from (x-step, y)
    tB = sid(x, y - step)          # inverse of bond 1 from (x, y-step)
    tF0 = sid(x + step, y)         # own bond 0
    tF1 = sid(x, y + step)         # own bond 1
    early_a = x >= step            # source (x-step, y) visited before (x, y)
    early_b = y >= step
    N = Lx * Ly
    tg = np.zeros((N, 4), dtype=np.int64)
    fw = np.zeros((N, 4), dtype=bool)
    # the four cases of which inverse links come before the site's own
    c11 = early_a & early_b
    c01 = ~early_a & early_b
    c10 = early_a & ~early_b
    c00 = ~early_a & ~early_b
    for mask, order in ((c11, ("A", "B", "F0", "F1")), (c01, ("B", "F0", "F1", "A")),
                        (c10, ("A", "F0", "F1", "B")), (c00, ("F0", "F1", "B", "A"))):
        for k, name in enumerate(order):
            t = {"A": tA, "B": tB, "F0": tF0, "F1": tF1}[name]
            tg[mask, k] = t[mask]
            fw[mask, k] = name.startswith("F")
    return tg, fw


def square_args_fast(model, L, T, J=-1.0, h=0.0, dmi=0.0, D=None, nthermal=10, nsweep=10, tau=0, algo=0,
                     frames=0, circuits=True, arrays=False):
    """The tuple of ``square_args`` (same values, same order) built with numpy
    array operations; for large lattices and served requests.  L even, >= 6.
    arrays=True returns numpy arrays in place of the inner tuples (for the
    C ABI, which takes buffers; the drop-in modules take tuples)."""
    if arrays:
        return _square_fast(model, L, T, J, h, dmi, D, nthermal, nsweep, tau, algo, frames, circuits, True)
    return _square_fast(model, L, T, J, h, dmi, D, nthermal, nsweep, tau, algo, frames, circuits, False)


def _square_fast(model, L, T, J, h, dmi, D, nthermal, nsweep, tau, algo, frames, circuits, arrays):
    if L < 6 or L % 2:
        return square_args(model, L, T, J=J, h=h, dmi=dmi, D=D, nthermal=nthermal, nsweep=nsweep, tau=tau,
                           algo=algo, frames=frames, circuits=circuits)
    T = max(T, 0.1)
    Lx = Ly = L
    N = L * L
    tg, fw = _square_link_order(Lx, Ly, 1)
    rtg, _ = _square_link_order(Lx, Ly, 2)
    x = np.repeat(np.arange(Lx), Ly)
    y = np.tile(np.arange(Ly), Lx)
    dirx = np.zeros((N, 4), dtype=bool)   # link along x (bond 0) or y (bond 1)
    sid = lambda a, b: (a % Lx) * Ly + (b % Ly)
    dirx[:] = (tg == sid(x + 1, y)[:, None]) | (tg == sid(x - 1, y)[:, None])
    chosen = (x % 2 == 0) & (y % 2 == 0)
    rorb = np.nonzero(chosen)[0]
    rcl = np.stack([sid(x, y), sid(x, y + 1), sid(x + 1, y), sid(x + 1, y + 1)], axis=1)[rorb]
    rlk = rtg[rorb]
    tau = N if tau <= 0 else tau
    cp = np.stack([np.arange(N), np.arange(N)], axis=1).reshape(-1)
    out = (lambda a: np.ascontiguousarray(a).reshape(-1)) if arrays else (lambda a: tuple(np.asarray(a).reshape(-1).tolist()))
    if model == "ising":
        K = J / T
        ls = np.full((N, 4), K)
        return (algo, out(np.ones(N)), nthermal, nsweep, tau, 4, out(np.full(N, 4)), out(ls), out(tg), out(cp), h / T,
                out(rorb), out(rcl), out(rlk), frames)
    bx = np.asarray(J9(J, J, J, xz=dmi, zx=-dmi), dtype=float) / T
    by = np.asarray(J9(J, J, J, yz=dmi, zy=-dmi), dtype=float) / T
    inv = lambda b: np.array([b[0], b[1], b[2], b[6], b[7], b[8], b[3], b[4], b[5]])
    ls = np.zeros((N, 4, 9))
    for k in range(4):
        ls[:, k, :] = np.where((dirx[:, k] & fw[:, k])[:, None], bx, 0) + \
            np.where((dirx[:, k] & ~fw[:, k])[:, None], inv(bx), 0) + \
            np.where((~dirx[:, k] & fw[:, k])[:, None], by, 0) + \
            np.where((~dirx[:, k] & ~fw[:, k])[:, None], inv(by), 0)
    Dv = np.asarray(D or [0, 0, 0], dtype=float) / T
    initD = np.tile(Dv, N)
    circ = np.zeros(0, dtype=np.int64)
    if circuits and model == "heisenberg":
        c = []
        for circuit in SQ_CIRCUITS:
            c.append(np.stack([sid(x + ov[0], y + ov[1]) for (o, ov) in circuit], axis=1))
        circ = np.stack(c, axis=1)
    ign = 0 if dmi != 0 else 1
    return (algo, out(np.ones(N)), out(initD), nthermal, nsweep, tau, 4, out(np.full(N, 4)), out(ls), out(tg),
            out(circ), out(cp), 1, N, out(np.arange(N)), 0.0, h / T, out(rorb), out(rcl), out(rlk), frames, ign)
