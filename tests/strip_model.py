"""A CPU model of the strip-wavefront lin_solve kernel (csrc/lssw.cuh), lane
by lane, used to check its schedule and index formulas against the oracle.

Block (b, g) owns strip b and the sweeps [g KG, g KG + nk). The model
follows the kernel's per-period order (chunk copies issued at the period's
start, imports, then each sweep warp's steps) and every shared-memory slot
carries the key of the value it holds and the first period in which a read
may see it; each read that the result depends on checks both, so a value
read before its barrier, or after its slot was reused, fails the check.
"""
import numpy as np

ROW, COL, PAS = 0, 1, 2
C_WALL, C_RL, C_RR, C_CD, C_CU, C_AD, C_CF = 1, 2, 4, 8, 16, 32, 64
F = np.float32


class Cfg:
    """The kernel's constants (lssw.cuh kSw*)."""
    Q = 4     # steps per period
    LG = 4    # steps between consecutive sweeps
    RD = 16   # diagonals per sweep ring
    RW = 36   # floats per ring row (positions -2 .. 33)
    PC = 128  # columns of the x0 / code rings
    PX = 32   # columns of the initial-x ring
    CH = 4    # columns per chunk copy
    AH = 5    # a row's chunk is issued AH periods before its first use period
    EDGE_RIGHT_FRAME = True  # the edge step sets an interior row's column S-1


def derive_codes(cells, S):
    """The per-cell boundary codes of the host's derive_codes."""
    N = S - 2
    wall = lambda i, j: cells[j * S + i] != 0
    code = np.zeros((S, S), np.uint8)
    rowfl = np.zeros(S, np.uint8)
    colfl = np.zeros(S, np.uint8)
    for j in range(S):
        for i in range(S):
            c = 0
            w = wall(i, j)
            if w:
                c |= C_WALL
            if not w and 1 <= i <= N and 1 <= j <= N:
                rowfl[j] = colfl[i] = 1
                if wall(i + 1, j):
                    c |= C_RR
                elif wall(i - 1, j):
                    c |= C_RL
                if wall(i, j - 1):
                    c |= C_CU
                elif wall(i, j + 1):
                    c |= C_CD
            if j >= 2 and j - 1 <= N and 1 <= i <= N and w and not wall(i, j - 1) \
                    and not wall(i, j - 2):
                c |= C_AD
            code[j, i] |= c
    for i in range(S):
        if colfl[i]:
            code[:, i] |= C_CF
    return code, rowfl, colfl


class Tracked:
    """Shared memory whose slots remember (key, first period a read may see it)."""

    def __init__(self, shape, dtype):
        self.v = np.zeros(shape, dtype)
        self.key = np.empty(shape, object)
        self.vfrom = np.full(shape, 1 << 30, np.int64)

    def write(self, idx, val, key, vfrom):
        self.v[idx] = val
        self.key[idx] = key
        self.vfrom[idx] = vfrom

    def read(self, idx, key, period, use, what):
        if use:
            if self.key[idx] != key:
                raise AssertionError(f"{what}: slot {idx} holds {self.key[idx]}, wanted {key}")
            if self.vfrom[idx] > period:
                raise AssertionError(f"{what}: {key} read in period {period}, valid from "
                                     f"{self.vfrom[idx]}")
        return self.v[idx]


def strips(S, K):
    return (S + 2 * (K - 1) + 31) // 32


def run(mode, x, x0, cells, S, P, K, a, c, G=1, cfg=Cfg):
    """One launch over K sweeps in G sweep groups: x with the last sweep's raw
    interior values (the caller then applies set_boundaries), and the number
    of (warp, step)s and of those on the fast path."""
    Q, LG, RD, PC, PX, AH, CH = cfg.Q, cfg.LG, cfg.RD, cfg.PC, cfg.PX, cfg.AH, cfg.CH
    N = S - 2
    a = F(a)
    cr = F(F(1.0) / F(c))
    code, rowfl, colfl = derive_codes(cells, S)
    xin = x.reshape(S, S).copy()
    xout = x.reshape(S, S).copy()
    x0g = x0.reshape(S, S)
    B = strips(S, K)
    KG = (K + G - 1) // G
    G = (K + KG - 1) // KG
    RE = S + 32
    TAG = 7
    edge = np.zeros((B, K, RE, 4), np.float32)  # [post30, -, uval31, post31]
    etag = np.zeros((B, K, RE, 4), np.int64)
    gexp = np.zeros((B, G, RE + 1, 36), np.float32)  # record d: positions -2..31 of d-1
    gtag = np.zeros((B, G, RE + 1, 36), np.int64)
    lanes = np.arange(32)
    steps = fast = 0

    def act(bb, k):
        j0 = 32 * bb - 2 * k
        return j0 <= S - 1 and j0 + 31 >= 0

    for b in range(B):
        for g in range(G):
            kF = g * KG
            nk = min(K, kF + KG) - kF
            jb = 32 * b - 2 * kF
            nrw = 32 + 2 * (nk - 1)
            rA = jb - 2 * (nk - 1)
            NP = (S + 32 + LG * (nk - 1) + Q - 1) // Q
            VR = Tracked((nk, RD, cfg.RW), np.float32)
            UI = Tracked((nk, RD), np.float32)
            VP = Tracked((RD, cfg.RW), np.float32)
            # rings with 4 padding columns that repeat columns 0 .. 3
            X0R = Tracked((nrw, PC + 4), np.float32)
            CR = Tracked((nrw, PC + 4), np.uint8)
            XR = Tracked((33, PX + 4), np.float32)

            def chunk_of(n, first):
                # row's 4-column chunk n is first read in the use period; a
                # CH-column copy goes out when n is a multiple of CH / 4 (and
                # in the first period, the copy under way)
                if n < 0 or 4 * n >= P:
                    return -1
                return n // (CH // 4) if n % (CH // 4) == 0 or first else -1

            def load_chunks(cp):
                u = cp + AH
                first = cp == -AH - 1
                for q in range(nrw):
                    r = rA + q
                    if r < 0 or r > S - 1:
                        continue
                    dr = jb - r
                    kmin = (dr + 1) >> 1 if dr > 0 else 0
                    m = chunk_of(u + ((dr - (LG + 2) * kmin + 3) >> 2), first)
                    if m < 0:
                        continue
                    for e in range(CH):
                        col = CH * m + e
                        for sc in ((col % PC,) if (CH * m) % PC else (col % PC, PC + e)):
                            # the frame rows' ring rows hold the frame rows of x
                            fr = r == 0 or r == S - 1
                            X0R.write((q, sc), (xin if fr else x0g)[r, col] if col < S else F(0),
                                      ("xf" if fr else "x0", r, col), u)
                            CR.write((q, sc), code[r, col] if col < S else 0,
                                     ("cd", r, col), u)
                if g == 0:
                    for q in range(33):
                        r = jb + q
                        if r > S - 1:
                            continue
                        m = chunk_of(u + 1 - ((q + 3) >> 2), first)
                        if m < 0:
                            continue
                        for e in range(CH):
                            col = CH * m + e
                            for sc in ((col % PX,) if (CH * m) % PX else (col % PX, PX + e)):
                                XR.write((q, sc), xin[r, col] if col < S else F(0),
                                         ("x", r, col), u)

            def halo_import(kk, cp):
                # the halo import warp: the words of use period cp + 1 (lane 0's
                # U ring, ring positions -2 / -1), one barrier before their use
                k = kF + kk
                if b == 0 or not act(b - 1, k):
                    return
                lo = (cp + 1) * Q - LG * kk - 1
                for dd in range(lo, lo + Q):
                    if dd < -1 or dd > S - 2:
                        continue
                    rec = dd + 32
                    assert (etag[b - 1, k, rec, [0, 2, 3]] == TAG).all(), ("halo", b, k, rec)
                    s = (dd + 1) % RD  # diagonal dd lives in slot dd + 1
                    VR.write((kk, s, 0), edge[b - 1, k, rec, 0], ("vr", k, dd, -2), cp + 1)
                    UI.write((kk, s), edge[b - 1, k, rec, 2], ("ui", k, dd), cp + 1)
                    VR.write((kk, s, 1), edge[b - 1, k, rec, 3], ("vr", k, dd, -1), cp + 1)

            def group_import(cp):
                if g == 0 or not act(b, kF):
                    return
                for d in range((cp + 1) * Q, (cp + 2) * Q):
                    if d < 0 or d > S + 31:
                        continue
                    assert (gtag[b, g - 1, d, :34] == TAG).all(), ("group", b, g, d)
                    for p in range(-2, 32):
                        VP.write((d % RD, p + 2), gexp[b, g - 1, d, p + 2],
                                 ("vr", kF - 1, d - 1, p), cp + 1)

            for cp in range(-AH - 1, 0):
                load_chunks(cp)
            for kk in range(nk):
                halo_import(kk, -1)
            group_import(-1)
            vcur = np.zeros((nk, 32), np.float32)
            vprev = np.zeros((nk, 32), np.float32)
            uprev = np.zeros((nk, 32), np.float32)
            cprev = np.zeros((nk, 32), np.uint8)
            for cp in range(NP):
                load_chunks(cp)
                group_import(cp)
                for kk in range(nk):
                    halo_import(kk, cp)
                    k = kF + kk
                    # a group's last sweep also runs (all lanes idle) when only the
                    # next group's first sweep has grid rows: it forwards the halo
                    if not act(b, k) and not (g < G - 1 and kk == nk - 1 and act(b, k + 1)):
                        continue
                    j0 = jb - 2 * kk
                    j = j0 + lanes
                    interior = (j >= 1) & (j <= N)
                    top, bot = j == 0, j == S - 1
                    idle = ~(interior | top | bot)
                    il = np.nonzero(interior)[0]
                    dF0 = il.max() + 2 if il.size else 1 << 30
                    dF1 = il.min() + N if il.size else -(1 << 30)
                    for t in range(Q):
                        d = cp * Q + t - LG * kk
                        if d < 0 or d > S + 31:
                            continue
                        steps += 1
                        i = d - lanes
                        jj, ii = np.clip(j, 0, S - 1), np.clip(i, 0, S - 1)
                        gsl = interior & (i >= 1) & (i <= N)
                        useR = gsl | (interior & (i == 0) & (mode == PAS) & (k > 0) &
                                      (rowfl[jj] != 0))
                        useD = gsl | (top & (i >= 0) & (i <= S - 1) & (mode == PAS) & (k > 0) &
                                      (colfl[ii] != 0))
                        R = np.zeros(32, np.float32)
                        D = np.zeros(32, np.float32)
                        for l in range(32):
                            if kk > 0:
                                sl = (kk - 1, d % RD)
                                R[l] = VR.read(sl + (l,), ("vr", k - 1, d - 1, l - 2), cp, useR[l], "R")
                                D[l] = VR.read(sl + (l + 1,), ("vr", k - 1, d - 1, l - 1), cp, useD[l], "D")
                            elif g > 0:
                                sl = (d % RD,)
                                R[l] = VP.read(sl + (l,), ("vr", k - 1, d - 1, l - 2), cp, useR[l], "R")
                                D[l] = VP.read(sl + (l + 1,), ("vr", k - 1, d - 1, l - 1), cp, useD[l], "D")
                            else:  # a period's columns from one base (no wrap)
                                dp = cp * Q - LG * kk
                                R[l] = XR.read((l, ((dp - l + 1) % PX) + t), ("x", j[l], i[l] + 1), cp,
                                               useR[l], "XR")
                                D[l] = XR.read((l + 1, ((dp - l) % PX) + t), ("x", j[l] + 1, i[l]), cp,
                                               useD[l], "XR")
                        U = np.empty(32, np.float32)
                        U[1:] = vcur[kk, :-1]
                        U[0] = UI.read((kk, d % RD), ("ui", k, d - 1), cp, bool(gsl[0]), "UI")
                        X0 = np.zeros(32, np.float32)
                        cd = np.zeros(32, np.uint8)
                        inr = (i >= 0) & (i <= S - 1)
                        useC = ((interior | bot) & (i >= 1) & (i <= N)) | ((top | bot) & inr)
                        for l in range(32):
                            rr = 2 * (nk - 1 - kk) + l
                            ci = ((cp * Q - LG * kk - l) % PC) + t  # a period's columns, one base
                            fr = bool(top[l] or bot[l])
                            X0[l] = X0R.read((rr, ci), ("xf" if fr else "x0", j[l], i[l]), cp,
                                             bool(gsl[l] or (fr and inr[l])), "X0")
                            cd[l] = CR.read((rr, ci), ("cd", j[l], i[l]), cp, bool(useC[l]), "CD")
                        with np.errstate(all="ignore"):
                            gs = ((X0 + a * (((R + vcur[kk]) + D) + U)) * cr).astype(np.float32)
                        vc = vcur[kk]
                        vnew = np.where(gsl, gs, vc)
                        i0 = interior & (i == 0)
                        vnew = np.where(i0 & (mode == PAS) & (k > 0) & (rowfl[jj] != 0), R,
                                        np.where(i0, xin[jj, 0], vnew))
                        vnew = np.where(interior & (i == S - 1), xin[jj, S - 1], vnew)
                        # frame rows: the frame value from the x0 ring, the column
                        # flag from the code
                        cfl = (cd & C_CF) != 0
                        vtop = np.where((mode == PAS) & (k > 0) & cfl, D, X0)
                        vnew = np.where(top & inr, vtop, vnew)
                        vnew = np.where(bot & inr, X0, vnew)
                        vnew = np.where(idle, F(0), vnew).astype(np.float32)
                        vdown = np.append(vnew[1:], vnew[31]).astype(np.float32)
                        im1 = i - 1
                        if mode == ROW:
                            pin = np.where(cprev[kk] & C_RR, -vnew,
                                           np.where(cprev[kk] & C_RL, -vprev[kk], vc))
                        elif mode == COL:
                            pin = np.where(cprev[kk] & C_CU, -uprev[kk],
                                           np.where(cprev[kk] & C_CD, -vdown, vc))
                        else:
                            pin = vc
                        post = np.where(interior & (im1 >= 1) & (im1 <= N), pin, vc)
                        pasrow = (mode == PAS) & (rowfl[jj] != 0)
                        post = np.where(interior & (im1 == 0) & pasrow, vnew, post)
                        post = np.where(interior & (im1 == S - 1) & pasrow, vprev[kk], post)
                        cfp = (mode == PAS) & ((cprev[kk] & C_CF) != 0) & (im1 >= 1) & (im1 <= N)
                        post = np.where(top & cfp, vdown, post)
                        post = np.where(bot & cfp, uprev[kk], post)
                        post = np.where(idle, F(0), post).astype(np.float32)
                        # the kernel's values: its fast step where every interior
                        # lane is at 2 <= i <= N, its edge step elsewhere. Both
                        # follow the general rules only where a later read needs
                        # them (an interior row's columns 0 .. S-1 and post values
                        # of columns 1 .. S-1, the frame rows' columns 0 .. S-1,
                        # the bottom row's post values of columns 1 .. N); the
                        # model carries the kernel's values on, so a read of any
                        # other value changes the result
                        edge_step = not (dF0 <= d <= dF1)
                        fast += not edge_step
                        pasr = (mode == PAS) & interior & (rowfl[jj] != 0)
                        if edge_step:
                            vL = np.where(pasr & (k > 0), R, np.where(interior, xin[jj, 0], F(0)))
                            xR = np.where(interior, xin[jj, S - 1], F(0))
                            ve = np.where(i == 0, vL, np.where(i == S - 1, xR, gs)
                                          if cfg.EDGE_RIGHT_FRAME else gs)
                        else:
                            ve = gs.copy()
                        fl = top | bot
                        ve = np.where(fl, np.where((mode == PAS) & top & (k > 0) & cfl, D, X0), ve)
                        ve = ve.astype(np.float32)
                        vde = np.append(ve[1:], ve[31]).astype(np.float32)
                        pe = vc.copy()
                        if mode == PAS:
                            pe = np.where(bot & ((cprev[kk] & C_CF) != 0), uprev[kk], pe)
                        if mode == ROW:
                            pe = np.where(interior, np.where(cprev[kk] & C_RR, -ve,
                                          np.where(cprev[kk] & C_RL, -vprev[kk], vc)), pe)
                        elif mode == COL:
                            pe = np.where(interior, np.where(cprev[kk] & C_CU, -uprev[kk],
                                          np.where(cprev[kk] & C_CD, -vde, vc)), pe)
                        elif edge_step:
                            pe = np.where(pasr & (im1 == S - 1), vprev[kk], pe)
                        pe = pe.astype(np.float32)
                        need_v = (interior | fl) & inr
                        need_p = (interior & (im1 >= 1) & (im1 <= S - 1)) | \
                                 (bot & (im1 >= 1) & (im1 <= N))
                        assert np.array_equal(ve[need_v].view(np.uint32),
                                              vnew[need_v].view(np.uint32))
                        assert np.array_equal(pe[need_p].view(np.uint32),
                                              post[need_p].view(np.uint32))
                        vnew, post = ve, pe
                        s = d % RD  # slot d holds diagonal d - 1
                        for l in range(32):
                            VR.write((kk, s, l + 2), post[l], ("vr", k, d - 1, l), cp + 1)
                        fixv = None
                        if mode == COL and (interior[0] or bot[0]) and 1 <= i[0] <= N \
                                and (cd[0] & C_AD):
                            fixv = -vnew[0]
                            VR.write((kk, s, 1), fixv, ("vr", k, d - 1, -1), cp + 1)
                        if b < B - 1 and d >= 1:
                            edge[b, k, d - 1, [0, 2, 3]] = (post[30], vc[31], post[31])
                            etag[b, k, d - 1, [0, 2, 3]] = TAG
                        if g < G - 1 and kk == nk - 1:
                            gexp[b, g, d, 2:34] = post
                            gexp[b, g, d, 0] = VR.v[kk, s, 0]
                            gexp[b, g, d, 1] = fixv if fixv is not None else VR.v[kk, s, 1]
                            gtag[b, g, d, :34] = TAG
                        if k == K - 1:
                            for l in np.nonzero(gsl)[0]:
                                xout[j[l], i[l]] = vnew[l]
                        vprev[kk] = vc
                        vcur[kk] = vnew
                        uprev[kk] = U
                        cprev[kk] = cd
    return xout.reshape(-1), steps, fast
