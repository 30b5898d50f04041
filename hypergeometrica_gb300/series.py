"""Hypergeometric series by binary splitting, with the partials on the GPU.

Mirrors src/binary-splitting.lisp:

  Series                  defstruct series (:16-35): integer functions a, b, p, q
                          of the series sum_k a(k)/b(k) * p(0)..p(k) / q(0)..q(k).
  Partial                 defstruct partial (:67-74): lower, upper, P, Q, B, R.
  partial_numerator /     partial-numerator, partial-denominator (:82-88).
  partial_denominator
  binary_split            binary-split (:123-133): split at floor((lower+upper)/2)
                          down to one-term base cases (:102-110), then combine
                          (:112-121) with seven mpz-* and one mpz-+.
  make_*_series           the series of :147-231 and src/pi.lisp:24-43.

The reference recurses one node at a time.  Here the same tree is evaluated
one height at a time: every node of a height combines at once.  Its five
independent products (P_l P_r, Q_l Q_r, B_l B_r, Q_r R_l, P_l R_r) and then
its two dependent ones (B_r (Q_r R_l), B_l (P_l R_r)) go to the
device-resident multiply service; R is one batched signed sum
(hg_add_batch_device) and P, Q, B get their sizes from one batched trim.
P, Q, B and R of every node stay in device memory, one arena per height,
until the parent has combined them.  For a series given by polynomials the
tree stops at nodes of at most 2^NODE_HEIGHT terms, each computed whole by
one device thread (hg_series_nodes_device); a range's partial is the same
integers however the range is split.  Because the tree is the reference's,
every partial it holds, not just the root, equals the reference's.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from fractions import Fraction
from typing import Callable

import numpy as np

from ._lib import HG_ERR_INCONSISTENT, HGError, check, load
from .mpz import NTT_MULTIPLY_THRESHOLD, digits_from_int, int_from_digits


def one(n: int) -> int:
    return 1


@dataclass(frozen=True)
class Series:
    """a, b, p, q as functions of k; `poly` optionally gives the same four as
    integer polynomials, ((c0, c1, ...), value at k = 0 or None) each, so that
    the base cases can be evaluated on the device."""

    a: Callable[[int], int] = one
    b: Callable[[int], int] = one
    p: Callable[[int], int] = one
    q: Callable[[int], int] = one
    poly: tuple | None = None


def _poly_series(a, b, p, q) -> Series:
    """A Series from four (coefficients low to high, value at 0 or None) pairs."""

    def fn(spec):
        coefs, zero = spec

        def f(n):
            if n == 0 and zero is not None:
                return zero
            acc = 0
            for c in reversed(coefs):
                acc = acc * n + c
            return acc

        return f

    return Series(a=fn(a), b=fn(b), p=fn(p), q=fn(q), poly=(a, b, p, q))


def _poly_bits(spec, n_max: int) -> int:
    coefs, zero = spec
    bound = sum(abs(c) * n_max ** i for i, c in enumerate(coefs))
    return max(bound.bit_length(), abs(zero or 0).bit_length())


def _device_leaves_fit(series: Series, upper: int) -> bool:
    if series.poly is None or upper > (1 << 62):
        return False
    for coefs, zero in series.poly:
        if len(coefs) > 8 or any(abs(c) >= 1 << 63 for c in coefs) or abs(zero or 0) >= 1 << 63:
            return False
    bits = [_poly_bits(spec, max(1, upper - 1)) for spec in series.poly]
    return max(bits) <= 254 and bits[2] + bits[0] <= 254


class DeviceInt:
    """A signed integer in device memory: limbs t[:size] (int64 tensor holding
    the 64-bit digits bit for bit; size excludes high zero limbs)."""

    __slots__ = ("sign", "t", "size")

    def __init__(self, sign: int, t, size: int):
        self.sign = 1 if size == 0 else int(sign)
        self.t = t
        self.size = int(size)

    @classmethod
    def from_int(cls, n: int) -> "DeviceInt":
        import torch

        d = digits_from_int(n)
        t = torch.from_numpy(d.view(np.int64).copy()).cuda() if d.size else torch.zeros(1, dtype=torch.int64,
                                                                                      device="cuda")
        return cls(-1 if n < 0 else 1, t, d.size)

    def to_int(self) -> int:
        if self.size == 0:
            return 0
        mag = int_from_digits(self.t[: self.size].cpu().numpy().view(np.uint64))
        return -mag if self.sign < 0 else mag

    def ptr(self) -> int:
        return self.t.data_ptr()


@dataclass
class Partial:
    lower: int
    upper: int
    p: DeviceInt
    q: DeviceInt
    b: DeviceInt
    r: DeviceInt


def partial_numerator(x: Partial) -> DeviceInt:
    return x.r


def partial_denominator(x: Partial, service=None) -> DeviceInt:
    """B * Q (partial-denominator)."""
    return multiply(x.b, x.q, service)


def multiply(x: DeviceInt, y: DeviceInt, service=None) -> DeviceInt:
    """mpz-* of two device integers (one product; through the service when
    given).  x is y squares (mpz-square's single forward transform)."""
    import torch

    from . import device as D

    square = x is y
    n = max(1, x.size + y.size)
    out = torch.empty(n, dtype=torch.int64, device="cuda")
    if x.size == 0 or y.size == 0:
        out.zero_()
        return DeviceInt(1, out, 0)
    xs, ys = x.t[: x.size], (None if square else y.t[: y.size])
    if not square and min(x.size, y.size) <= NTT_MULTIPLY_THRESHOLD:
        # mpz-*'s dispatch: a smaller operand of at most 100 limbs goes to the
        # quadratic method (src/multiply.lisp:37-42), here on the device
        big, small = (xs, ys) if x.size >= y.size else (ys, xs)
        D.mul_schoolboy(big, small, out)
        sizes = trim_sizes([(out, n)])
        return DeviceInt(x.sign * y.sign, out, int(sizes[0]))
    if service is not None:
        torch.cuda.current_stream().synchronize()
        (t,) = service.submit([(xs, ys, out)])
        service.wait(t)
    elif square:
        D.sqr(xs, out)
        D.sync()
    else:
        D.mul(xs, ys, out)
        D.sync()
    sizes = trim_sizes([(out, n)])
    return DeviceInt(x.sign * y.sign, out, int(sizes[0]))


def mpz_expt_device(a, n: int, service=None) -> DeviceInt:
    """mpz-expt (src/multiply.lisp:77-79) with the operand and every partial
    power in device memory: f-expt's left-to-right binary powering
    (:51-75), squaring through mpz-square."""
    from .mpz import f_expt

    x = a if isinstance(a, DeviceInt) else DeviceInt.from_int(a)
    return f_expt(x, n, DeviceInt.from_int(1), lambda u, v: multiply(u, v, service))


def trim_sizes(vecs) -> np.ndarray:
    """mpz-size of (tensor, length) pairs on the device (hg_trim_batch_device)."""
    import torch

    rec = np.array([[t.data_ptr(), n] for t, n in vecs], dtype=np.uint64).reshape(-1, 2)
    return _trim_records(rec)


SMALL_MAX_LIMBS = 64  # HG_SMALL_MAX_LIMBS
# Tree nodes of height <= NODE_HEIGHT (at most 2^NODE_HEIGHT terms) whose
# parent is higher are computed whole on the device (hg_series_nodes_device)
# instead of level by level.
NODE_HEIGHT = 6


def _multiply_records(rec: np.ndarray, service) -> None:
    """Run (n, 6) hg_product records: by the one-thread-per-product schoolbook
    kernel when every operand has at most SMALL_MAX_LIMBS limbs (on the torch
    stream), else through the service (a callable returning it), waiting for
    them."""
    import torch

    if rec.shape[0] == 0:
        return
    if int(rec[:, 1].max()) <= SMALL_MAX_LIMBS and int(rec[:, 3].max()) <= SMALL_MAX_LIMBS:
        rec = np.ascontiguousarray(rec, dtype=np.uint64)
        st = torch.cuda.current_stream()
        check(load().hg_mul_small_batch_device(rec.ctypes.data_as(ctypes.c_void_p), rec.shape[0], st.cuda_stream))
        return
    torch.cuda.current_stream().synchronize()
    svc = service()
    svc.submit_records(rec)
    svc.wait_all()


def _trim_records(rec: np.ndarray) -> np.ndarray:
    import torch

    n = rec.shape[0]
    if n == 0:
        return np.zeros(0, dtype=np.int64)
    sizes = torch.empty(n, dtype=torch.int64, device="cuda")
    rec = np.ascontiguousarray(rec, dtype=np.uint64)
    st = torch.cuda.current_stream()
    check(load().hg_trim_batch_device(rec.ctypes.data_as(ctypes.c_void_p), n, sizes.data_ptr(), st.cuda_stream))
    return sizes.cpu().numpy()


def _sum_records(rec: np.ndarray) -> np.ndarray:
    """hg_add_batch_device on (n, 8) records; returns (n, 2) [sign, size]."""
    import torch

    n = rec.shape[0]
    res = torch.empty(2 * n, dtype=torch.int64, device="cuda")
    rec = np.ascontiguousarray(rec, dtype=np.uint64)
    st = torch.cuda.current_stream()
    check(load().hg_add_batch_device(rec.ctypes.data_as(ctypes.c_void_p), n, res.data_ptr(), st.cuda_stream))
    return res.cpu().numpy().reshape(n, 2)


# ---- the recursion tree -------------------------------------------------


def _tree(lower: int, upper: int, stop: int = 1):
    """The nodes of binary-split's recursion over [lower, upper), top down,
    not expanding nodes of at most `stop` terms: arrays lo, hi, left child,
    right child (-1 for unexpanded nodes), height (= ceil(log2(hi - lo)) for
    this split)."""
    lo = [np.array([lower], dtype=np.int64)]
    hi = [np.array([upper], dtype=np.int64)]
    first = [0]
    lefts, rights = [], []
    cur_lo, cur_hi, nid = lo[0], hi[0], 1
    while True:
        inner = (cur_hi - cur_lo) > stop
        left = np.full(cur_lo.size, -1, dtype=np.int64)
        right = np.full(cur_lo.size, -1, dtype=np.int64)
        k = int(inner.sum())
        if k:
            left[inner] = nid + 2 * np.arange(k)
            right[inner] = left[inner] + 1
        lefts.append(left)
        rights.append(right)
        if not k:
            break
        l, u = cur_lo[inner], cur_hi[inner]
        m = (l + u) // 2
        cur_lo = np.stack([l, m], axis=1).reshape(-1)
        cur_hi = np.stack([m, u], axis=1).reshape(-1)
        first.append(nid)
        lo.append(cur_lo)
        hi.append(cur_hi)
        nid += 2 * k
    lo, hi = np.concatenate(lo), np.concatenate(hi)
    left, right = np.concatenate(lefts), np.concatenate(rights)
    # ceil(log2(span)) = bit length of span - 1: the binary exponent frexp
    # returns, exact because span - 1 < 2^53.
    height = np.frexp((hi - lo - 1).astype(np.float64))[1].astype(np.int64)
    return lo, hi, left, right, height


def _pack(values):
    """Signs, (n, w) little-endian limbs and trimmed sizes of Python ints."""
    n = len(values)
    signs = np.fromiter((-1 if v < 0 else 1 for v in values), dtype=np.int64, count=n)
    mags = [abs(v) for v in values]
    w = max(1, max(((m.bit_length() + 63) // 64 for m in mags), default=1))
    buf = b"".join(m.to_bytes(8 * w, "little") for m in mags)
    limbs = np.frombuffer(buf, dtype="<u8").astype(np.uint64).reshape(n, w)
    nz = limbs != 0
    sizes = np.where(nz.any(axis=1), w - np.argmax(nz[:, ::-1], axis=1), 0).astype(np.int64)
    return signs, limbs, sizes, w


def _footprint_bound(total_limbs: int) -> int:
    """Workspace of the largest product whose operands hold total_limbs limbs."""
    n = 1 << max(1, (max(1, total_limbs) - 1).bit_length())
    return 2 * 3 * n * 8


def binary_split(series: Series, lower: int, upper: int, service=None, timings: list | None = None) -> Partial:
    """binary-split (src/binary-splitting.lisp:123-133) on the GPU.  When
    `timings` is a list, one (height, nodes, seconds of products, seconds of
    sums and trims) record per height is appended to it, after a
    ("tree", nodes, seconds) and a ("leaves", count, seconds) record for the
    tree's base nodes (whole nodes of up to 2^NODE_HEIGHT terms, or single
    terms for a series without polynomials)."""
    import time

    import torch

    from . import device as D

    if upper <= lower:
        raise ValueError("binary-split needs upper > lower")
    t_start = time.perf_counter()
    whole = _device_leaves_fit(series, upper)
    # Whole nodes: the tree stops at nodes of at most 2^NODE_HEIGHT terms.
    lo, hi, left, right, height = _tree(lower, upper, (1 << NODE_HEIGHT) if whole else 1)
    nn = lo.size
    if timings is not None:
        timings.append(("tree", int(nn), time.perf_counter() - t_start))
    t_start = time.perf_counter()
    leaves = np.flatnonzero(left < 0)
    ptr = np.zeros((4, nn), dtype=np.uint64)
    size = np.zeros((4, nn), dtype=np.int64)
    sign = np.ones((4, nn), dtype=np.int64)
    H = int(height.max())
    h_first, arena_key = 1, 0  # the first height combined level by level; key of the base arena
    root_off = None  # the root's arena and the offsets of its P, Q, B, R
    if whole:
        # The unexpanded nodes (height <= h0, parent higher): one device
        # thread each folds the node's terms (the same integers as the
        # reference's recursion below that node).  Their parents are at
        # heights h0 + 1 and h0 + 2.
        h0 = NODE_HEIGHT
        cut = leaves
        arena0, ss, width = _device_nodes(series, lo[cut], hi[cut], upper)
        base = arena0.data_ptr()
        nc = np.uint64(cut.size)
        cidx = np.arange(cut.size, dtype=np.uint64)
        for j in range(4):
            ptr[j, cut] = base + np.uint64(8 * width) * (np.uint64(j) * nc + cidx)
            sign[j, cut] = ss[j, :, 0]
            size[j, cut] = ss[j, :, 1]
        if (size[:, cut] < 0).any():
            raise HGError(HG_ERR_INCONSISTENT, "series node partial exceeded its width bound")
        leaf_limbs = int(size[:, cut].sum())
        h_first, arena_key = h0 + 1, h0
        if cut[0] == 0:  # the root itself
            root_off = (arena0, [j * cut.size * width for j in range(4)])
    else:
        # binary-split-base-case=1 (:102-110): P = p(k), Q = q(k), B = b(k), R = p(k) a(k)
        ks = lo[leaves].tolist()
        pv = [series.p(k) for k in ks]
        vals = [pv, [series.q(k) for k in ks], [series.b(k) for k in ks],
                [pk * series.a(k) for pk, k in zip(pv, ks)]]
        base_off = 0
        packed = [_pack(v) for v in vals]
        leaf_limbs = sum(int(pk[2].sum()) for pk in packed)
        arena0 = torch.from_numpy(np.concatenate([pk[1].reshape(-1) for pk in packed]).view(np.int64)).cuda()
        base = arena0.data_ptr()
        for j, (sg, limbs, sz, w) in enumerate(packed):
            ptr[j, leaves] = base + 8 * (base_off + w * np.arange(leaves.size, dtype=np.uint64))
            size[j, leaves] = sz
            sign[j, leaves] = sg
            base_off += w * leaves.size
        if H == 0:
            root_off = (arena0, [int((ptr[j, 0] - np.uint64(base)) // np.uint64(8)) for j in range(4)])
    arenas = {arena_key: arena0}
    del arena0
    if timings is not None:
        timings.append(("leaves", int(leaves.size), time.perf_counter() - t_start))
    own = []

    def get_service():
        """The caller's service, else one opened on first use, sized for the
        largest product the tree can form."""
        if service is not None:
            return service
        if not own:
            ws = max(64 << 20, _footprint_bound(2 * leaf_limbs))
            own.append(D.Service(workspace_bytes=2 * ws, slots=2))
        return own[0]

    torch.cuda.synchronize()
    try:
        order = np.argsort(height, kind="stable")
        bounds = np.searchsorted(height[order], np.arange(H + 2))
        for h in range(h_first, H + 1):
            idx = order[bounds[h]: bounds[h + 1]]
            L, R = left[idx], right[idx]
            k = idx.size
            sL, sR = size[:, L], size[:, R]
            gL, gR = sign[:, L], sign[:, R]
            pL, pR = ptr[:, L], ptr[:, R]
            szP, szQ, szB = sL[0] + sR[0], sL[1] + sR[1], sL[2] + sR[2]
            szT1, szT2 = sR[1] + sL[3], sL[0] + sR[3]
            szT3, szT4 = sR[2] + szT1, sL[2] + szT2
            szR = np.maximum(szT3, szT4) + 1
            keep = [szP, szQ, szB, szR]
            tmp = [szT1, szT2, szT3, szT4]
            keep_off = _offsets(keep)
            tmp_off = _offsets(tmp)
            arena = torch.empty(max(1, int(sum(int(s.sum()) for s in keep))), dtype=torch.int64, device="cuda")
            scratch = torch.empty(max(1, int(sum(int(s.sum()) for s in tmp))), dtype=torch.int64, device="cuda")
            ab, sb_ = np.uint64(arena.data_ptr()), np.uint64(scratch.data_ptr())
            aP, aQ, aB, aR = (ab + np.uint64(8) * o for o in keep_off)
            t1, t2, t3, t4 = (sb_ + np.uint64(8) * o for o in tmp_off)
            stage1 = D.product_records(
                np.concatenate([pL[0], pL[1], pL[2], pR[1], pL[0]]),
                np.concatenate([sL[0], sL[1], sL[2], sR[1], sL[0]]),
                np.concatenate([pR[0], pR[1], pR[2], pL[3], pR[3]]),
                np.concatenate([sR[0], sR[1], sR[2], sL[3], sR[3]]),
                np.concatenate([aP, aQ, aB, t1, t2]),
                np.concatenate([szP, szQ, szB, szT1, szT2]))
            t0 = time.perf_counter()
            _multiply_records(stage1, get_service)
            stage2 = D.product_records(np.concatenate([pR[2], pL[2]]), np.concatenate([sR[2], sL[2]]),
                                       np.concatenate([t1, t2]), np.concatenate([szT1, szT2]),
                                       np.concatenate([t3, t4]), np.concatenate([szT3, szT4]))
            _multiply_records(stage2, get_service)
            t1 = time.perf_counter()
            sgT1, sgT2 = gR[1] * gL[3], gL[0] * gR[3]
            sgT3, sgT4 = gR[2] * sgT1, gL[2] * sgT2
            sums = np.stack([t3, szT3.astype(np.uint64), t4, szT4.astype(np.uint64), aR, szR.astype(np.uint64),
                             sgT3.astype(np.int64).view(np.uint64), sgT4.astype(np.int64).view(np.uint64)], axis=1)
            res = _sum_records(sums)
            trims = np.stack([np.concatenate([aP, aQ, aB]),
                              np.concatenate([szP, szQ, szB]).astype(np.uint64)], axis=1)
            tsz = _trim_records(trims)
            if timings is not None:
                timings.append((h, int(k), t1 - t0, time.perf_counter() - t1))
            ptr[0, idx], ptr[1, idx], ptr[2, idx], ptr[3, idx] = aP, aQ, aB, aR
            size[0, idx], size[1, idx], size[2, idx] = tsz[:k], tsz[k: 2 * k], tsz[2 * k:]
            size[3, idx] = res[:, 1]
            sign[0, idx], sign[1, idx], sign[2, idx] = gL[0] * gR[0], gL[1] * gR[1], gL[2] * gR[2]
            sign[3, idx] = res[:, 0]
            arenas[h] = arena
            if h == H:
                root_off = (arena, [int(o[0]) for o in keep_off])
            del scratch
            arenas.pop(h - 2, None)
    finally:
        for svc in own:
            svc.close()

    def dev_int(j: int) -> DeviceInt:
        arena, o = root_off
        return DeviceInt(int(sign[j, 0]), arena[o[j]:], int(size[j, 0]))

    return Partial(lower, upper, dev_int(0), dev_int(1), dev_int(2), dev_int(3))


def _device_leaves(series: Series, lower: int, upper: int):
    """hg_series_leaves_device: ((4 * count * 4) limb arena, (4, count, 2) signs and sizes)."""
    import torch

    count = upper - lower
    limbs = torch.empty(16 * count, dtype=torch.int64, device="cuda")
    ss = torch.empty(8 * count, dtype=torch.int64, device="cuda")
    st = torch.cuda.current_stream()
    check(load().hg_series_leaves_device(_polys(series), lower, count, limbs.data_ptr(), ss.data_ptr(),
                                         st.cuda_stream))
    return limbs, ss.cpu().numpy().reshape(4, count, 2)


def _device_nodes(series: Series, lo: np.ndarray, hi: np.ndarray, upper: int):
    """hg_series_nodes_device for the node ranges [lo, hi): ((4 * n * width)
    limb arena, (4, n, 2) signs and sizes, width).  The width bounds every
    value: with s_v the limbs of the largest |v(k)|, k < upper, and
    S = s_p + s_q + s_b + s_r + 1, a node of m terms has |R| < 2^(64 m S)
    and P, Q, B, B P below that."""
    import torch

    n = int(lo.size)
    bits = [_poly_bits(spec, max(1, upper - 1)) for spec in series.poly]  # a, b, p, q
    lim = lambda b: max(1, -(-b // 64))  # noqa: E731
    S = lim(bits[2]) + lim(bits[3]) + lim(bits[1]) + lim(bits[2] + bits[0]) + 1
    width = max(8, S * int((hi - lo).max()) + 1)
    ranges = torch.from_numpy(np.stack([lo, hi], axis=1).reshape(-1).astype(np.int64)).cuda()
    limbs = torch.empty(4 * n * width, dtype=torch.int64, device="cuda")
    scratch = torch.empty(2 * n * width, dtype=torch.int64, device="cuda")
    ss = torch.empty(8 * n, dtype=torch.int64, device="cuda")
    st = torch.cuda.current_stream()
    check(load().hg_series_nodes_device(_polys(series), ranges.data_ptr(), n, width, limbs.data_ptr(),
                                        ss.data_ptr(), scratch.data_ptr(), st.cuda_stream))
    out = ss.cpu().numpy().reshape(4, n, 2)
    del scratch, ranges
    return limbs, out, width


def _polys(series: Series):
    from ._lib import HgPoly

    polys = (HgPoly * 4)()
    for j, (coefs, zero) in enumerate(series.poly):
        for i, c in enumerate(coefs):
            polys[j].coef[i] = c
        polys[j].degree = len(coefs) - 1
        polys[j].has_zero_value = 0 if zero is None else 1
        polys[j].zero_value = 0 if zero is None else zero
    return polys


def _offsets(sizes_list):
    """Start offsets of consecutive blocks: sizes_list[0] for every node, then
    sizes_list[1], ..."""
    out, base = [], 0
    for s in sizes_list:
        s = np.asarray(s, dtype=np.int64)
        c = np.cumsum(s) - s + base
        out.append(c.astype(np.uint64))
        base += int(s.sum())
    return out


# ---- series of the reference ---------------------------------------------


def make_exp_series(x) -> Series:
    """make-exp-series (src/binary-splitting.lisp:147-155): e^x for rational x."""
    x = Fraction(x)
    num, den = x.numerator, x.denominator
    return _poly_series(a=((1,), None), b=((1,), None), p=((num,), 1), q=((0, den), 1))


def make_e_series() -> Series:
    """make-e-series (:157-161)."""
    return _poly_series(a=((1,), None), b=((1,), None), p=((1,), None), q=((0, 1), 1))


def make_ramanujan_series() -> Series:
    """make-ramanujan-series (:174-193): p = 32k^3 - 48k^2 + 22k - 3, q = k^3 396^4 / 8."""
    return _poly_series(a=((1103, 26390), None), b=((1,), None), p=((-3, 22, -48, 32), 1),
                        q=((0, 0, 0, 396 ** 4 // 8), 1))


def make_catalan_series() -> Series:
    """make-catalan-series (:213-223)."""
    return _poly_series(a=((1,), None), b=((1, 2), None), p=((0, 1), 1), q=((2, 4), 1))


def make_apery_series() -> Series:
    """make-apery-series (:226-231): q = 32 (2k + 1)^5 expanded."""
    return _poly_series(a=((77, 250, 205), None), b=((2,), None), p=((0, 0, 0, 0, 0, -1), 1),
                        q=((32, 320, 1280, 2560, 2560, 1024), None))


CHUD_A, CHUD_B, CHUD_C = 13591409, 545140134, 640320
CHUD_PREFACTOR = 10  # pi/10 (src/pi.lisp:17-22)
CHUD_BITS_PER_TERM = math.log2(151931373056000)
CHUD_DECIMALS_PER_TERM = math.log10(151931373056000)


def make_chudnovsky_series() -> Series:
    """make-chudnovsky-series (src/pi.lisp:24-43), for pi/10: a = 10 (A + B k),
    b = 8 C / 12, p = -72k^3 + 108k^2 - 46k + 5, q = k^3 C^3 / 24."""
    return _poly_series(a=((CHUD_A * CHUD_PREFACTOR, CHUD_B * CHUD_PREFACTOR), None),
                        b=(((8 * CHUD_C) // 12,), None), p=((5, -46, 108, -72), 1),
                        q=((0, 0, 0, CHUD_C ** 3 // 24), 1))


def chudnovsky_terms(prec_bits: int) -> int:
    """num-terms of mpd-pi (src/pi.lisp:53-56): 2 + floor(guard / bits-per-term)."""
    guard = prec_bits + 64
    return 2 + math.floor(guard / CHUD_BITS_PER_TERM)
