"""CPU model of the three-block vertex pass's shared-memory tiles
(k_vertex_mn_split: one 32-plane-wave chunk, one 128-row tile), written from
the address arithmetic of k_vertex_mn.cu: the X gathers (rows = local field x
band, K = Re / Im parts of the chunk's plane waves, 128-byte swizzle), the Y
copies of the three column blocks c, b1 c, b2 c (64-byte swizzle: 32-wide
atoms, LBO = 512 bytes between atoms, SBO = one 8-row K group of hi and lo
atoms), and the 24 MMAs of a chunk: per K step of 16 the three split products
Xl.Yh + Xh.Yl + Xh.Yh into Re D, and the same against the other K half of Y,
negated where X holds real parts, into Im D.  Checks that every shared-memory
element is written at most once and that Re D and Im D equal
D((G,a), b) = sum_i x_a(G,i) conj(y_b(i)) for all three blocks.  The GPU tests
check the kernel itself against the oracle; this pins the layout and the
sign reasoning on the CPU."""
import numpy as np
import pytest


def _tile(NBY, XB, nbp, xs, ys, seed):
    rng = np.random.default_rng(seed)
    NB = 3
    NYN = NB * NBY
    AB = 512                       # bytes of one 64-byte-swizzle atom (32 columns x 8 K rows)
    NTA = (NYN + 31) // 32         # atoms along N of one half (hi or lo) of Y
    XH = 64 * 128 * 2              # one half (hi or lo) of X
    YKG = 2 * NTA * AB             # Y bytes per group of 8 K rows: hi atoms, then lo atoms
    YLO = NTA * AB
    STAGE = 2 * XH + 8 * YKG
    GPT = 128 // XB
    npos = 64
    # coefficient planes [position][re_hi, im_hi, re_lo, im_lo][band]
    Xpl = rng.standard_normal((npos, 4, nbp))
    Ypl = [rng.standard_normal((32, 4, nbp)) for _ in range(NB)]  # c, b1 c, b2 c
    pos = rng.integers(-1, npos, size=(GPT, 32))  # Gfast positions (G, plane wave), -1 none
    sm = np.zeros(STAGE // 2)
    written = np.zeros(STAGE // 2, dtype=np.int32)

    def put(addr, vals):
        assert addr % 16 == 0 and 0 <= addr and addr + 16 <= STAGE
        sm[addr // 2: addr // 2 + 8] = vals
        written[addr // 2: addr // 2 + 8] += 1

    def pad8(v):
        return np.concatenate([v, np.zeros(8 - len(v))]) if len(v) < 8 else v

    # X copies: copy thread ptid -> plane waves xpw and xpw + 16, rows 8 xj .. 8 xj + 7
    for ptid in range(256):
        xpw, xj = ptid >> 4, ptid & 15
        xrow = 8 * xj
        xg, xb0 = xrow // XB, xrow % XB
        ok = xg < GPT and xs + xb0 < nbp
        for pw in (xpw, xpw + 16):
            xoff = (pw >> 3) * 2048 + (xj >> 3) * 1024 + (pw & 7) * 128 + (((xj & 7) ^ (pw & 7)) << 4)
            p = pos[xg, pw] if ok else -1
            for u4 in range(4):
                d = xoff + (u4 >> 1) * XH + (u4 & 1) * 8192
                put(d, pad8(Xpl[p, u4, xs + xb0: xs + xb0 + 8]) if p >= 0 else np.zeros(8))

    # Y copies: e = ptid + 256 v over 2 halves x 64 K rows x NYN / 8 chunks
    YCH = NYN // 8
    for e in range(128 * YCH):
        line, j = e // YCH, e % YCH
        half, kk = line >> 6, line & 63
        part, pw = kk >> 5, kk & 31
        col = 8 * j
        u = 2 * half + part
        blk = col // NBY
        band = ys + col - blk * NBY
        dst = 2 * XH + (kk >> 3) * YKG + half * YLO + (col >> 5) * 512 + (kk & 7) * 64 + \
            ((((col >> 3) & 3) ^ ((kk & 7) >> 1)) << 4)
        put(dst, pad8(Ypl[blk][pw, u, band: band + 8]) if band < nbp else np.zeros(8))
    assert written.max() <= 1

    # operand reads: MN-major 128-byte swizzle (X) and 64-byte swizzle (Y)
    def operand_sw128(start, lbo, sbo, MN):
        A = np.zeros((MN, 16))
        for mn in range(MN):
            for k in range(16):
                off = start + (mn // 64) * lbo + (k // 8) * sbo + (k % 8) * 128
                a = (off + ((((mn % 64) // 8) ^ (k % 8)) * 16) + (mn % 8) * 2) // 2
                assert 0 <= a < STAGE // 2
                A[mn, k] = sm[a]
        return A

    def operand_sw64(start, lbo, sbo, MN):
        B = np.zeros((MN, 16))
        for mn in range(MN):
            for k in range(16):
                off = start + (mn // 32) * lbo + (k // 8) * sbo + (k % 8) * 64
                a = (off + ((((mn % 32) // 8) ^ ((k % 8) >> 1)) * 16) + (mn % 8) * 2) // 2
                assert 0 <= a < STAGE // 2
                B[mn, k] = sm[a]
        return B

    Dr = np.zeros((128, NYN))
    Di = np.zeros((128, NYN))
    for ks in range(4):
        xh = ks * 4096
        xl = xh + XH
        Ah, Al = operand_sw128(xh, 1024, 2048, 128), operand_sw128(xl, 1024, 2048, 128)
        yh = 2 * XH + ks * 2 * YKG
        Bh, Bl = operand_sw64(yh, AB, YKG, NYN), operand_sw64(yh + YLO, AB, YKG, NYN)
        Dr += Al @ Bh.T + Ah @ Bl.T + Ah @ Bh.T
        ih = 2 * XH + (ks ^ 2) * 2 * YKG
        Ih, Il = operand_sw64(ih, AB, YKG, NYN), operand_sw64(ih + YLO, AB, YKG, NYN)
        sign = -1.0 if ks < 2 else 1.0  # the instruction descriptor's negate-B bit
        Di += sign * (Al @ Ih.T + Ah @ Il.T + Ah @ Ih.T)

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
        blk = n // NBY
        band = ys + n - blk * NBY
        if band < nbp:
            h, l = split(Ypl[blk])
            Yh[n], Yl[n] = h[:, band], l[:, band]
    ref = Xl @ Yh.conj().T + Xh @ Yl.conj().T + Xh @ Yh.conj().T
    return Dr, Di, ref


@pytest.mark.parametrize("NBY,XB,nbp,xs,ys", [
    (32, 32, 30, 0, 0),    # the 30-band current pass: one 32-band window on both sides
    (32, 24, 40, 8, 16),   # 24 gathered rows per field (rows 120-127 padding), offset windows
    (16, 16, 80, 64, 48),  # 16-band windows of an 80-band basis
])
def test_split_vertex_tile_layout(NBY, XB, nbp, xs, ys):
    re, im, ref = _tile(NBY, XB, nbp, xs, ys, seed=NBY + XB + nbp)
    scale = max(np.abs(ref).max(), 1.0)
    assert np.abs(re - ref.real).max() <= 1e-12 * scale
    assert np.abs(im - ref.imag).max() <= 1e-12 * scale
