"""CPU model of the tensor-core S0 accumulation's operand tiles for one
32-transition chunk, written from the address arithmetic of k_accum_tc.cu:
the pre-split B tiles of k_presplit_ws (rows G' of B1 = [Re b | Im b] and of
B2 = [-Im b | Re b], the four 16-byte groups of a row on neighbouring tasks),
the A tile the formation warps write (row G = [Re a | Im a] with a = w M), the
128-byte swizzle (16-byte chunk c of row r at position c ^ (r % 8)) and the
K-major descriptor reads of the four K steps (start + 32 bytes per step).
Checks that the three split products D = Ah.Bl + Al.Bh + Ah.Bh over
[B1; B2] give Re and Im of sum_t w_t M_t(G) conj(M2_t(G')) — the complex S0
contribution of the chunk for one frequency row."""
import numpy as np

TT, GA, GB = 32, 128, 96


def _split(x):
    """fp16 hi + lo of float32 values, as split8<true> forms them."""
    x = np.asarray(x, dtype=np.float32)
    hi = x.astype(np.float16)
    lo = (x - hi.astype(np.float32)).astype(np.float16)
    return hi.astype(np.float64), lo.astype(np.float64)


def _st16(tile, row, chunk, vals):
    tile[row, ((chunk ^ (row & 7)) * 8):((chunk ^ (row & 7)) * 8 + 8)] = vals


def _read(tile, rows, ks):
    """K-major SW128 operand of K step ks: rows x 16 values."""
    out = np.zeros((rows, 16))
    for r in range(rows):
        for kk in range(16):
            k = 16 * ks + kk
            pos = ((k // 8) ^ (r & 7)) * 8 + k % 8
            out[r, kk] = tile[r, pos]
    return out


def test_accumulation_tile_layout():
    rng = np.random.default_rng(3)
    nlf = 91
    M = (rng.standard_normal((TT, nlf)) + 1j * rng.standard_normal((TT, nlf))).astype(np.complex64)
    w = rng.standard_normal(TT).astype(np.float32)
    # B tiles (k_presplit_ws<complex>): task -> row = rem >> 2, grp = rem & 3
    B = {h: np.zeros((2 * GB, 64)) for h in ("hi", "lo")}
    for rem in range(GB * 4):
        row, grp = rem >> 2, rem & 3
        if row < nlf:
            b = M[grp * 8: grp * 8 + 8, row]
        else:
            b = np.zeros(8, dtype=np.complex64)
        rh, rl = _split(b.real)
        ih, il = _split(b.imag)
        _st16(B["hi"], row, grp, rh)
        _st16(B["lo"], row, grp, rl)
        _st16(B["hi"], row, 4 + grp, ih)
        _st16(B["lo"], row, 4 + grp, il)
        _st16(B["hi"], GB + row, grp, -ih)   # split(-x) = -split(x)
        _st16(B["lo"], GB + row, grp, -il)
        _st16(B["hi"], GB + row, 4 + grp, rh)
        _st16(B["lo"], GB + row, 4 + grp, rl)
    # A tile (formation warps): row = e >> 3, ch = e & 7; a = w (hi + lo of b) re-split
    A = {h: np.zeros((GA, 64)) for h in ("hi", "lo")}
    for e in range(nlf * 8):
        row, ch = e >> 3, e & 7
        part, grp = ch >> 2, ch & 3
        b = M[grp * 8: grp * 8 + 8, row]
        bh, bl = _split(b.imag if part else b.real)
        x = (bh + bl).astype(np.float32) * w[grp * 8: grp * 8 + 8]
        ah, al = _split(x)
        _st16(A["hi"], row, ch, ah)
        _st16(A["lo"], row, ch, al)
    D = np.zeros((GA, 2 * GB))
    for ks in range(4):
        Ah, Al = _read(A["hi"], GA, ks), _read(A["lo"], GA, ks)
        Bh, Bl = _read(B["hi"], 2 * GB, ks), _read(B["lo"], 2 * GB, ks)
        D += Ah @ Bl.T + Al @ Bh.T + Ah @ Bh.T
    ref = (M.T * w) @ M.conj()  # [G, G'] = sum_t w_t M_t(G) conj(M_t(G'))
    ref = ref.astype(np.complex128)
    scale = np.abs(ref).max()
    assert np.abs(D[:nlf, :nlf] - ref.real).max() <= 2e-6 * scale
    assert np.abs(D[:nlf, GB:GB + nlf] - ref.imag).max() <= 2e-6 * scale
    assert np.abs(D[nlf:, :]).max() == 0 and np.abs(D[:, nlf:GB]).max() == 0


def test_accumulation_with_a_in_tensor_memory():
    """The A tile formed in tensor memory (shapes whose TMEM columns fit): row
    G of the tile in lane G, the 16-bit K values of chunk ch (8 values) in the
    four 32-bit columns 4 ch .. 4 ch + 3, two per column (even K in the low
    half), hi in columns 0-31 and lo in 32-63 of the slot; the MMA of K step
    ks reads columns 8 ks .. 8 ks + 7 of hi and of lo.  Against the B tiles of
    k_presplit_ws read as the K-major descriptor reads them, the three split
    products give the chunk's complex S0 contribution, as the shared-memory A
    tile does."""
    rng = np.random.default_rng(5)
    nlf = 91
    M = (rng.standard_normal((TT, nlf)) + 1j * rng.standard_normal((TT, nlf))).astype(np.complex64)
    w = rng.standard_normal(TT).astype(np.float32)
    B = {h: np.zeros((2 * GB, 64)) for h in ("hi", "lo")}
    for rem in range(GB * 4):
        row, grp = rem >> 2, rem & 3
        b = M[grp * 8: grp * 8 + 8, row] if row < nlf else np.zeros(8, dtype=np.complex64)
        rh, rl = _split(b.real)
        ih, il = _split(b.imag)
        _st16(B["hi"], row, grp, rh)
        _st16(B["lo"], row, grp, rl)
        _st16(B["hi"], row, 4 + grp, ih)
        _st16(B["lo"], row, 4 + grp, il)
        _st16(B["hi"], GB + row, grp, -ih)
        _st16(B["lo"], GB + row, grp, -il)
        _st16(B["hi"], GB + row, 4 + grp, rh)
        _st16(B["lo"], GB + row, 4 + grp, rl)
    # TMEM slot: lanes x 64 columns of two 16-bit values (column col holds K = 2 col, 2 col + 1)
    tm = np.zeros((128, 64, 2))
    for lane in range(128):
        for ch in range(8):
            part, grp = ch >> 2, ch & 3
            if lane < nlf:
                b = M[grp * 8: grp * 8 + 8, lane]
                bh, bl = _split(b.imag if part else b.real)
                x = (bh + bl).astype(np.float32) * w[grp * 8: grp * 8 + 8]
            else:
                x = np.zeros(8, dtype=np.float32)
            ah, al = _split(x)
            for q in range(4):  # column 4 ch + q holds K values 8 ch + 2q, 8 ch + 2q + 1
                tm[lane, 4 * ch + q] = ah[2 * q: 2 * q + 2]
                tm[lane, 32 + 4 * ch + q] = al[2 * q: 2 * q + 2]
    D = np.zeros((128, 2 * GB))
    for ks in range(4):
        Ah = tm[:, 8 * ks: 8 * ks + 8].reshape(128, 16)
        Al = tm[:, 32 + 8 * ks: 32 + 8 * ks + 8].reshape(128, 16)
        Bh, Bl = _read(B["hi"], 2 * GB, ks), _read(B["lo"], 2 * GB, ks)
        D += Ah @ Bl.T + Al @ Bh.T + Ah @ Bh.T
    ref = ((M.T * w) @ M.conj()).astype(np.complex128)
    scale = np.abs(ref).max()
    assert np.abs(D[:nlf, :nlf] - ref.real).max() <= 2e-6 * scale
    assert np.abs(D[:nlf, GB:GB + nlf] - ref.imag).max() <= 2e-6 * scale
    assert np.abs(D[nlf:, :]).max() == 0
