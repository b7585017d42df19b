"""Seeded synthetic operands with the value mix the benchmark configurations
describe (no dataset is involved; these stand in for the reference's
published vector sets at their sizes).

Every element is a dense little-endian encoding held as uint32 words: an
(n, W) array per operand, W = 1, 2, 4, 8 for fp32/64/128/256.

The mix, per operand:
  * 90% normals: random sign, random fraction, unbiased exponent uniform
    in [-64, 64];
  * 10% specials, spread over: +-0, random subnormals, +-inf, quiet NaNs
    with a random payload, signalling NaNs with a random non-zero payload,
    and values within 2 ulp of the largest normal.
Per element, on top of that:
  * exact-cancellation triples: a and b with significands of at most p/2
    bits, so a*b is exact, and c = -(a*b);
  * halfway cases (with ties=True): a*b with exactly p+1 significant bits
    and its last bit set (a tie for MUL and for FMA with c = +-0), and
    a + c with c exactly half an ulp of a (a tie for ADD/SUB).
"""
import numpy as np

GEOM = {0: (8, 23), 1: (11, 52), 2: (15, 112), 3: (19, 236)}   # (exp_w, man_w)


def words(fmt):
    return (1, 2, 4, 8)[fmt]


def geometry(fmt):
    expw, manw = GEOM[fmt]
    return dict(expw=expw, manw=manw, prec=manw + 1, bias=(1 << (expw - 1)) - 1,
                width=32 * words(fmt), W=words(fmt), es=manw - 32 * (words(fmt) - 1))


def to_int(wrow):
    v = 0
    for i, w in enumerate(wrow):
        v |= int(w) << (32 * i)
    return v


def from_int(v, W):
    return [(v >> (32 * i)) & 0xFFFFFFFF for i in range(W)]


def encode(fmt, sign, sig, e2):
    """The encoding of (-1)^sign * sig * 2^e2, which must be an exactly
    representable normal (sig > 0)."""
    g = geometry(fmt)
    p = g["prec"]
    L = sig.bit_length()
    assert 0 < L <= p
    sh = p - L
    sig <<= sh
    e2 -= sh
    biased = e2 + (p - 1) + g["bias"]
    assert 1 <= biased <= (1 << g["expw"]) - 2, biased
    return (sign << (g["width"] - 1)) | (biased << g["manw"]) | (sig & ((1 << g["manw"]) - 1))


def _rand_bits(rng, k):
    """A random k-bit integer with its top bit set."""
    v = int.from_bytes(rng.bytes((k + 7) // 8), "little") & ((1 << k) - 1)
    return v | (1 << (k - 1))


def _specials(fmt, rng, m):
    """m special encodings as an (m, W) uint32 array."""
    g = geometry(fmt)
    W, es, expw, manw = g["W"], g["es"], g["expw"], g["manw"]
    out = rng.integers(0, 1 << 32, size=(m, W), dtype=np.uint64).astype(np.uint32)
    cat = rng.integers(0, 6, size=m)
    sign = rng.integers(0, 2, size=m).astype(np.uint32)
    top = out[:, W - 1] & np.uint32((1 << es) - 1)              # fraction bits in the top word
    expmax = (1 << expw) - 1
    quiet_word, quiet_bit = (manw - 1) >> 5, (manw - 1) & 31
    for k in range(6):
        sel = cat == k
        if not sel.any():
            continue
        if k == 0:                                               # +-0
            out[sel, :] = 0
            out[sel, W - 1] = sign[sel] << 31
        elif k == 1:                                             # subnormal
            out[sel, W - 1] = (sign[sel] << 31) | top[sel]
            out[sel, 0] |= 1                                     # keep it non-zero
        elif k == 2:                                             # +-inf
            out[sel, :] = 0
            out[sel, W - 1] = (sign[sel] << 31) | np.uint32(expmax << es)
        elif k in (3, 4):                                        # qNaN / sNaN
            out[sel, W - 1] = (sign[sel] << 31) | np.uint32(expmax << es) | top[sel]
            if k == 3:
                out[sel, quiet_word] |= np.uint32(1 << quiet_bit)
            else:
                out[sel, quiet_word] &= np.uint32(~(1 << quiet_bit) & 0xFFFFFFFF)
                out[sel, 0] |= 1                                 # payload non-zero
        else:                                                    # within 2 ulp of max normal
            out[sel, :] = 0xFFFFFFFF
            out[sel, W - 1] = (sign[sel] << 31) | np.uint32((expmax - 1) << es) | np.uint32((1 << es) - 1)
            dec = rng.integers(0, 3, size=int(sel.sum())).astype(np.uint32)
            out[sel, 0] -= dec
    return out


def gen_operands(fmt, n, seed, special_frac=0.10, exp_range=64, triples_frac=0.015,
                 ties=False):
    """(a, b, c): three (n, W) uint32 arrays."""
    g = geometry(fmt)
    W, es = g["W"], g["es"]
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(3):
        x = rng.integers(0, 1 << 32, size=(n, W), dtype=np.uint64).astype(np.uint32)
        sign = rng.integers(0, 2, size=n).astype(np.uint32)
        e = (g["bias"] + rng.integers(-exp_range, exp_range + 1, size=n)).astype(np.uint32)
        x[:, W - 1] = (x[:, W - 1] & np.uint32((1 << es) - 1)) | (e << np.uint32(es)) | (sign << np.uint32(31))
        m = rng.random(n) < special_frac
        cnt = int(m.sum())
        if cnt:
            x[m] = _specials(fmt, rng, cnt)
        ops.append(x)
    a, b, c = ops
    p = g["prec"]
    # exact-cancellation triples
    nt = int(n * triples_frac)
    if nt:
        idx = rng.choice(n, size=nt, replace=False)
        h = p // 2
        for i in idx:
            sa, sb = _rand_bits(rng, h) | 1, _rand_bits(rng, h) | 1
            ea, eb = int(rng.integers(-40, 40)), int(rng.integers(-40, 40))
            s1, s2 = int(rng.integers(0, 2)), int(rng.integers(0, 2))
            a[i] = from_int(encode(fmt, s1, sa, ea), W)
            b[i] = from_int(encode(fmt, s2, sb, eb), W)
            c[i] = from_int(encode(fmt, 1 - (s1 ^ s2), sa * sb, ea + eb), W)
    if ties and 2 * nt <= n and nt:
        idx = rng.choice(n, size=2 * nt, replace=False)
        for j, i in enumerate(idx):
            if j % 2 == 0:
                # a*b with exactly p+1 bits, the last one set: a tie for MUL
                # and for FMA with c = +-0
                for _ in range(64):
                    ka = int(rng.integers(2, p))
                    sa = _rand_bits(rng, ka) | 1
                    sb = _rand_bits(rng, p + 2 - ka) | 1
                    if (sa * sb).bit_length() == p + 1:
                        break
                else:
                    continue
                a[i] = from_int(encode(fmt, int(rng.integers(0, 2)), sa, int(rng.integers(-30, 30))), W)
                b[i] = from_int(encode(fmt, int(rng.integers(0, 2)), sb, int(rng.integers(-30, 30))), W)
                c[i] = 0
                c[i, W - 1] = np.uint32(int(rng.integers(0, 2)) << 31)      # +-0
            else:
                # c exactly half an ulp of a: a tie for ADD and SUB
                ea = int(rng.integers(-30, 30))
                a[i] = from_int(encode(fmt, int(rng.integers(0, 2)), _rand_bits(rng, p), ea), W)
                c[i] = from_int(encode(fmt, int(rng.integers(0, 2)), 1, ea - 1), W)
                b[i] = from_int(encode(fmt, 0, 1, 0), W)                    # 1.0
    return a, b, c


def to_bytes(x):
    """(n, W) uint32 -> the dense little-endian byte string the ABI takes."""
    return np.ascontiguousarray(x, dtype="<u4").tobytes()


def from_bytes(buf, fmt):
    return np.frombuffer(buf, dtype="<u4").reshape(-1, words(fmt))


def encode_double(fmt, x):
    """The exact encoding of the binary64 value x in format fmt (fmt >= 1:
    every double is representable in binary64, 128 and 256)."""
    import struct
    bits = struct.unpack("<Q", struct.pack("<d", float(x)))[0]
    g = geometry(fmt)
    sign, e, frac = bits >> 63, (bits >> 52) & 0x7FF, bits & ((1 << 52) - 1)
    if e == 0 and frac == 0:
        return sign << (g["width"] - 1)
    if e == 0x7FF:
        raise ValueError("not finite")
    if e == 0:                                   # subnormal double
        sig, e2 = frac, -1074
    else:
        sig, e2 = frac | (1 << 52), e - 1023 - 52
    return encode(fmt, sign, sig, e2)


def hard_rows(fmt, m, seed):
    """m operand rows (a, b, c), each (m, W) uint32, that are all hard cases
    of the value mix: the first half exact-cancellation triples (a*b exact,
    c = -(a*b)); then, alternately, a*b with exactly p+1 significant bits and
    its last bit set with c = +-0 (a tie for MUL and FMA) and a + c with c
    exactly half an ulp of a and b = 1.0 (a tie for ADD and SUB). Planted
    into device-generated arrays (plant()), they give those arrays the mix
    gen_operands() gives host arrays, at sizes where building every row on
    the host would take minutes."""
    g = geometry(fmt)
    W, p = g["W"], g["prec"]
    rng = np.random.default_rng(seed)
    a = np.zeros((m, W), np.uint32)
    b = np.zeros((m, W), np.uint32)
    c = np.zeros((m, W), np.uint32)
    h = p // 2
    for i in range(m):
        if i < m // 2:
            sa, sb = _rand_bits(rng, h) | 1, _rand_bits(rng, h) | 1
            ea, eb = int(rng.integers(-40, 40)), int(rng.integers(-40, 40))
            s1, s2 = int(rng.integers(0, 2)), int(rng.integers(0, 2))
            a[i] = from_int(encode(fmt, s1, sa, ea), W)
            b[i] = from_int(encode(fmt, s2, sb, eb), W)
            c[i] = from_int(encode(fmt, 1 - (s1 ^ s2), sa * sb, ea + eb), W)
        elif i % 2 == 0:
            for _ in range(64):
                ka = int(rng.integers(2, p))
                sa = _rand_bits(rng, ka) | 1
                sb = _rand_bits(rng, p + 2 - ka) | 1
                if (sa * sb).bit_length() == p + 1:
                    break
            a[i] = from_int(encode(fmt, int(rng.integers(0, 2)), sa, int(rng.integers(-30, 30))), W)
            b[i] = from_int(encode(fmt, int(rng.integers(0, 2)), sb, int(rng.integers(-30, 30))), W)
            c[i, W - 1] = np.uint32(int(rng.integers(0, 2)) << 31)              # +-0
        else:
            ea = int(rng.integers(-30, 30))
            a[i] = from_int(encode(fmt, int(rng.integers(0, 2)), _rand_bits(rng, p), ea), W)
            c[i] = from_int(encode(fmt, int(rng.integers(0, 2)), 1, ea - 1), W)
            b[i] = from_int(encode(fmt, 0, 1, 0), W)                            # 1.0
    return a, b, c


def plant(fmt, tensors, n, seed, frac=0.045, rows=8192):
    """Write hard_rows() (cycled) over a fraction `frac` of the n elements of
    three device operand tensors (torch, n*W int32 each) at seeded distinct
    positions; returns the positions (sorted int64)."""
    import torch
    W = words(fmt)
    hr = hard_rows(fmt, rows, seed)
    rng = np.random.default_rng(seed + 1)
    k = min(n, int(n * frac))
    if k == 0:
        return np.zeros(0, np.int64)
    pos = np.sort(rng.choice(n, size=k, replace=False)).astype(np.int64)
    which = rng.integers(0, rows, size=k)
    ti = torch.from_numpy(pos).to(tensors[0].device)
    for t, h in zip(tensors, hr):
        src = torch.from_numpy(np.ascontiguousarray(h[which]).view(np.int32)).to(t.device)
        t.view(-1, W).index_copy_(0, ti, src)
    return pos
