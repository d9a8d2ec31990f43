"""CPU model of the tensor-core vertex kernel's shared-memory tiles (one
32-plane-wave chunk, one 128-row tile), written from the address arithmetic of
k_vertex_mn.cu: the X gathers (rows = local field x band, K = Re / Im parts of
the chunk's plane waves), the Y copies with their y' images, and the operand
reads of the MN-major 128-byte-swizzle descriptors (LBO = stride between
64-element atoms, SBO = stride between 8-row K groups).  Checks that every
shared-memory element is written at most once and that the twelve MMAs of a
chunk (Xl.Yh + Xh.Yl + Xh.Yh per K step of 16) give Re and Im of
D((G,a), b) = sum_i x_a(G,i) conj(y_b(i)) for the bands of both column blocks
(c and b(i) c for current vertices).  The GPU tests check the same kernel
against the oracle; this pins the layout reasoning on the CPU."""
import numpy as np
import pytest


def _tile(NBY, CURRENT, XB, nbp, xs, ys, seed):
    rng = np.random.default_rng(seed)
    NYN = (2 if CURRENT else 1) * NBY
    NTA = (2 * NYN + 63) // 64
    XH, YKG, YLO, N2 = 64 * 128 * 2, NTA * 2048, NTA * 1024, 64 * NTA
    STAGE = 2 * XH + 8 * YKG
    GPT = 128 // XB
    npos = 64
    # coefficient planes [position][re_hi, im_hi, re_lo, im_lo][band]
    Xpl = rng.standard_normal((npos, 4, nbp))
    Ypl = rng.standard_normal((32, 4, nbp))
    Ybt = rng.standard_normal((32, 4, nbp))
    pos = rng.integers(-1, npos, size=(GPT, 32))  # Gfast positions (G, plane wave), -1 none
    sm = np.zeros(STAGE // 2)
    written = np.zeros(STAGE // 2, dtype=np.int32)

    def put(addr, vals):
        assert addr % 16 == 0 and 0 <= addr and addr + 16 <= STAGE
        sm[addr // 2: addr // 2 + 8] = vals
        written[addr // 2: addr // 2 + 8] += 1

    def get(addr):
        return sm[addr // 2: addr // 2 + 8].copy()

    def pad8(v):
        return np.concatenate([v, np.zeros(8 - len(v))]) if len(v) < 8 else v

    # X copies: thread tid -> plane wave xpw, rows 8 xj .. 8 xj + 7, four planes
    for tid in range(512):
        xpw, xj = tid >> 4, tid & 15
        xrow = 8 * xj
        xg, xb0 = xrow // XB, xrow % XB
        ok = xg < GPT and xs + xb0 < nbp
        xoff = (xpw >> 3) * 2048 + (xj >> 3) * 1024 + (xpw & 7) * 128 + (((xj & 7) ^ (xpw & 7)) << 4)
        p = pos[xg, xpw] if ok else -1
        for u4 in range(4):
            d = xoff + (u4 >> 1) * XH + (u4 & 1) * 8192
            put(d, pad8(Xpl[p, u4, xs + xb0: xs + xb0 + 8]) if p >= 0 else np.zeros(8))

    # Y copies: e = tid + 512 v over 2 halves x 64 K rows x NYN / 8 chunks; each
    # copied chunk also lands as its y' image (row kk ^ 32, column NYN + col,
    # negated for the imaginary part)
    def yoff(half, kk, col):
        return 2 * XH + (kk >> 3) * YKG + half * YLO + (col >> 6) * 1024 + (kk & 7) * 128 + \
            ((((col >> 3) & 7) ^ (kk & 7)) << 4)

    YCH = NYN // 8
    for e in range(128 * YCH):
        line, j = e // YCH, e % YCH
        half, kk = line >> 6, line & 63
        part, pw = kk >> 5, kk & 31
        col = 8 * j
        bblk = CURRENT and col >= NBY
        band = ys + (col - NBY if bblk else col)
        src = pad8((Ybt if bblk else Ypl)[pw, 2 * half + part, band: band + 8]) if band < nbp else np.zeros(8)
        put(yoff(half, kk, col), src)
        w = get(yoff(half, kk, col))
        put(yoff(half, kk ^ 32, NYN + col), -w if part else w)
    assert written.max() <= 1

    # operand reads of an MN-major SW128 descriptor
    def operand(start, lbo, sbo, MN):
        A = np.zeros((MN, 16))
        for mn in range(MN):
            for k in range(16):
                off = start + (mn // 64) * lbo + (k // 8) * sbo + (k % 8) * 128
                chunk = ((mn % 64) // 8) ^ (k % 8)
                a = (off + chunk * 16 + (mn % 8) * 2) // 2
                assert 0 <= a < STAGE // 2
                A[mn, k] = sm[a]
        return A

    D = np.zeros((128, N2))
    for ks in range(4):
        xh = ks * 4096
        xl = xh + XH
        yh = 2 * XH + ks * 2 * YKG
        yl = yh + YLO
        Ah, Al = operand(xh, 1024, 2048, 128), operand(xl, 1024, 2048, 128)
        Bh, Bl = operand(yh, 1024, YKG, N2), operand(yl, 1024, YKG, N2)
        D += Al @ Bh.T + Ah @ Bl.T + Ah @ Bh.T

    # direct: the same three split products in complex arithmetic
    def split(pl):
        return pl[..., 0, :] + 1j * pl[..., 1, :], pl[..., 2, :] + 1j * pl[..., 3, :]

    Xh = np.zeros((128, 32), complex)
    Xl = np.zeros((128, 32), complex)
    for r in range(128):
        g, a = r // XB, r % XB
        if g >= GPT or xs + a >= nbp:
            continue
        for i in range(32):
            if pos[g, i] >= 0:
                h, l = split(Xpl[pos[g, i]])
                Xh[r, i], Xl[r, i] = h[xs + a], l[xs + a]
    Yh = np.zeros((NYN, 32), complex)
    Yl = np.zeros((NYN, 32), complex)
    for n in range(NYN):
        bblk = CURRENT and n >= NBY
        band = ys + (n - NBY if bblk else n)
        if band < nbp:
            h, l = split(Ybt if bblk else Ypl)
            Yh[n], Yl[n] = h[:, band], l[:, band]
    ref = Xl @ Yh.conj().T + Xh @ Yl.conj().T + Xh @ Yh.conj().T
    return D[:, :NYN], D[:, NYN:2 * NYN], ref


@pytest.mark.parametrize("NBY,CURRENT,XB,nbp,xs,ys", [
    (32, True, 32, 32, 0, 0),      # current vertices, one 32-band window
    (16, True, 16, 80, 64, 48),    # current, 16-band windows of an 80-band basis
    (32, False, 8, 32, 0, 8),      # charge, occupied side gathered (8 rows per field)
    (64, False, 32, 184, 32, 88),  # charge, 64-band column window
    (48, False, 16, 80, 0, 8),     # charge, 48-band column window
])
def test_vertex_tile_layout(NBY, CURRENT, XB, nbp, xs, ys):
    re, im, ref = _tile(NBY, CURRENT, XB, nbp, xs, ys, seed=NBY + XB + nbp)
    scale = max(np.abs(ref).max(), 1.0)
    assert np.abs(re - ref.real).max() <= 1e-12 * scale
    assert np.abs(im - ref.imag).max() <= 1e-12 * scale
