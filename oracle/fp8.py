"""CPU restatement of libptg's FP8 (e4m3) tensor storage and of the operands of its FP8
MTTKRP -- TEST INFRASTRUCTURE ONLY (the checker of the GPU path, never part of it).

The reference stores tensors in FP64 only (include/Tensor.hpp:36-101); FP8 storage is this
project's own format, so this file restates the project's definition, step for step in the
same FP32 arithmetic, for bit-exact comparison:

  storage   slab s = index of the last mode; scale_s = 2^k, k the smallest integer with
            max_slab |x| <= 448 * 2^k; v = float32(x) * 2^-k; the e4m3 neighbours of v are
            spaced sp = 2^-9 below 2^-6, else 2^(floor(log2 |v|) - 3); with y = |v| / sp and
            t = y - floor(y), v rounds away from zero iff t * 2^24 > u, u = the top 24 bits
            of the splitmix64 finaliser of (position * 0x9E3779B97F4A7C15 +
            0x632BE59BD9B4E019), position = the entry's index in the ColMajor FP64 source.
  operand   a Khatri-Rao value (the FP32 product of factor entries, modes after the solved
            one first, then the modes before it) times the slab scale (when the slab index
            is contracted) times c_r = 2^k with smax * prod_f max_i |A_f(i, r)| * c_r in
            (128, 256]; hi = e4m3 round-to-nearest-even of a, lo = that of 16 (a - hi);
            the kernel contracts hi and lo and returns (X.hi + X.lo / 16) / c_r.
"""
from __future__ import annotations

import numpy as np

E4M3_MAX = 448.0


def dither(pos: np.ndarray) -> np.ndarray:
    """24-bit dither of each source position (uint64 arithmetic wraps like the device's)."""
    z = np.asarray(pos, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15) + np.uint64(0x632BE59BD9B4E019)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z ^= z >> np.uint64(31)
    return (z >> np.uint64(40)).astype(np.uint32)


def _spacing(a: np.ndarray) -> np.ndarray:
    """Spacing of the e4m3 grid at |v| = a (float32)."""
    _, e = np.frexp(a)                       # a = m 2^e, m in [0.5, 1): floor(log2 a) = e - 1
    sp = np.ldexp(np.float32(1.0), (e - 1 - 3).astype(np.int32)).astype(np.float32)
    return np.where(a < np.float32(2.0 ** -6), np.float32(2.0 ** -9), sp).astype(np.float32)


def _code_of(r: np.ndarray, neg: np.ndarray) -> np.ndarray:
    """e4m3 code of the non-negative e4m3 values r, with the sign bits of neg."""
    small = r < np.float32(2.0 ** -6)
    m, e = np.frexp(np.where(small, np.float32(1.0), r))
    E = (e - 1).astype(np.int64)
    mant = ((m * 2.0 - 1.0) * 8.0).astype(np.int64)
    code = np.where(small, (r * np.float32(512.0)).astype(np.int64), ((E + 7) << 3) | mant)
    return (code | np.where(neg, 0x80, 0)).astype(np.uint8)


def encode_sr(v: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Stochastic rounding of float32 v (|v| <= 448) to e4m3 codes with dither u."""
    v = np.asarray(v, dtype=np.float32)
    a = np.abs(v)
    sp = _spacing(a)
    y = (a / sp).astype(np.float32)          # exact: sp is a power of two
    fl = np.floor(y)
    up = (y - fl) * np.float32(16777216.0) > np.asarray(u).astype(np.float32)
    r = ((fl + up.astype(np.float32)) * sp).astype(np.float32)
    return _code_of(r, np.signbit(v))


def rne(a: np.ndarray) -> np.ndarray:
    """float32 -> nearest e4m3 value (ties to even, saturating at +-448), as float32."""
    a = np.asarray(a, dtype=np.float32)
    mag = np.abs(a)
    sp = _spacing(mag)
    r = (np.rint(mag / sp) * sp).astype(np.float32)
    r = np.minimum(r, np.float32(E4M3_MAX))
    return np.where(np.signbit(a), -r, r).astype(np.float32)


def decode(codes: np.ndarray) -> np.ndarray:
    """Exact value of e4m3 codes (float64)."""
    c = np.asarray(codes, dtype=np.int64)
    e, m = (c >> 3) & 15, c & 7
    mag = np.where(e == 0, m * 2.0 ** -9, np.ldexp(1.0 + m / 8.0, (e - 7).astype(np.int32)))
    return np.where(c & 0x80, -mag, mag)


def scale_exp(mx: np.ndarray) -> np.ndarray:
    """k of the slab scale 2^k: the smallest k with mx <= 448 * 2^k (0 for mx = 0)."""
    mx = np.asarray(mx, dtype=np.float64)
    f, E = np.frexp(mx)
    k = np.where(f <= 0.875, E - 9, E - 8)
    k = np.where(mx > 0, k, 0)
    return np.clip(k, -126, 127).astype(np.int32)


def encode_tensor(X: np.ndarray):
    """X: float64 array of shape dims (ColMajor semantics).  Returns the codes (flat,
    ColMajor, unpadded), the slab scales (float32, one per index of the last mode) and the
    stored values scale * decode(code) in the shape of X."""
    dims = X.shape
    flat = np.asarray(X, dtype=np.float64).reshape(-1, order="F")
    nslab = dims[-1]
    per = flat.size // nslab
    mx = np.abs(flat.reshape(nslab, per)).max(axis=1)
    k = scale_exp(mx)
    scales = np.ldexp(np.float32(1.0), k).astype(np.float32)
    inv = np.ldexp(np.float32(1.0), -k).astype(np.float32)
    v = (flat.astype(np.float32).reshape(nslab, per) * inv[:, None]).astype(np.float32).reshape(-1)
    codes = encode_sr(v, dither(np.arange(flat.size, dtype=np.uint64)))
    vals = (decode(codes).reshape(nslab, per) * scales[:, None].astype(np.float64)).reshape(-1)
    return codes, scales, vals.reshape(dims, order="F")


def _kr_side(factors, modes):
    """FP32 Khatri-Rao rows over `modes` (first mode fastest), products in the kernel's
    order 1 * A_first * A_next ..."""
    R = factors[0].shape[1]
    out = np.ones((1, R), dtype=np.float32)
    for k in modes:
        A = np.asarray(factors[k], dtype=np.float32)
        out = (out[None, :, :] * A[:, None, :]).reshape(-1, R).astype(np.float32)
    return out


def col_scales(factors, mode, slab_max_scale):
    """c_r of the kernel: smax * prod_f max_i |A_f(i, r)| in (128, 256] after scaling."""
    N = len(factors)
    R = factors[0].shape[1]
    m = np.full(R, float(slab_max_scale), dtype=np.float64)
    for f in list(range(mode)) + list(range(mode + 1, N)):
        m = m * np.abs(np.asarray(factors[f], dtype=np.float32)).max(axis=0).astype(np.float64)
    fr, E = np.frexp(m)
    k = np.where(fr == 0.5, 9 - E, 8 - E)
    k = np.where((m > 0) & np.isfinite(m), np.clip(k, -120, 120), 0)
    return np.ldexp(np.float32(1.0), k.astype(np.int32)).astype(np.float32)


def mttkrp(codes: np.ndarray, scales: np.ndarray, dims, factors, mode: int) -> np.ndarray:
    """The FP8 MTTKRP with every operand rounded exactly as the kernel rounds it, summed in
    FP64 (the only remaining difference to the GPU is its FP32 accumulation)."""
    N = len(dims)
    R = factors[0].shape[1]
    last = N - 1
    Ka = _kr_side(factors, list(range(mode + 1, N)))     # [S, R]
    Kb = _kr_side(factors, list(range(mode)))            # [P, R]
    P, S, Q = Kb.shape[0], Ka.shape[0], dims[mode]
    slab_in_q = mode == last
    smax = 1.0 if slab_in_q else float(scales.max())
    c = col_scales(factors, mode, smax)
    if slab_in_q:
        row_sc = np.ones(S, dtype=np.float32)
    else:
        div = int(np.prod(dims[mode + 1:last])) if mode + 1 < last else 1
        row_sc = scales[np.arange(S) // div].astype(np.float32)
    V = (Ka[None, :, :] * Kb[:, None, :]).astype(np.float32)             # [P, S, R]
    A = (V * (row_sc[None, :, None] * c[None, None, :])).astype(np.float32)
    hi = rne(A)
    lo = rne(((A - hi) * np.float32(16.0)).astype(np.float32))
    B = hi.astype(np.float64) + lo.astype(np.float64) / 16.0
    Xc = decode(codes).reshape(S, Q, P).transpose(2, 1, 0)                # [P, Q, S] raw codes
    M = np.einsum("pqs,psr->qr", Xc, B, optimize=True) / c.astype(np.float64)[None, :]
    if slab_in_q:
        M = M * scales.astype(np.float64)[:, None]
    return M
