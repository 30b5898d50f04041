"""Binary splitting on the GPU (series.binary_split) and the batched signed
sums and trims it is built from, against the oracle.

Integers throughout: every comparison is exact.  Small and medium ranges
compare P, Q, B, R with the oracle's recursion on Python integers; the
Chudnovsky ranges of 2^22 and 2^24-bit pi compare them modulo primes with
the oracle's closed forms (a size-independent check).
"""

import numpy as np
import pytest

import series_oracle as O
from hypergeometrica_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _as_int(limbs, sign=1):
    from hypergeometrica_gb300.mpz import int_from_digits

    v = int_from_digits(limbs)
    return -v if sign < 0 else v


def _dev(a):
    import torch

    a = np.ascontiguousarray(a, dtype=np.uint64)
    if a.size == 0:
        return torch.zeros(1, dtype=torch.int64, device="cuda"), 0
    return torch.from_numpy(a.view(np.int64).copy()).cuda(), a.size


def _cases(sizes=(0, 1, 2, 7, 2047, 2048, 2049, 5000, 20000), count=60, seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        na = int(rng.choice(sizes))
        nb = int(rng.choice(sizes))
        a = W.limbs(10 * k + 1, na)
        b = W.limbs(10 * k + 2, nb)
        kind = k % 6
        if kind == 1:  # long carry chains
            a = np.full(na, np.uint64(2**64 - 1))
            b = np.zeros(nb, dtype=np.uint64)
            if nb:
                b[0] = 1
        elif kind == 2 and na:  # equal magnitudes
            b = a.copy()
        elif kind == 3 and na and nb:  # equal tops, differ low
            b = a.copy()
            b[0] ^= np.uint64(1)
        elif kind == 4 and na > 1:  # borrow chains: a = 2^(64(n-1)), b = 1
            a = np.zeros(na, dtype=np.uint64)
            a[-1] = 1
            b = np.ones(1, dtype=np.uint64)
        signs = [(1, 1), (1, -1), (-1, 1), (-1, -1)][k % 4]
        out.append((a, b, *signs))
    return out


LARGE_SUM_SIZES = (0, 1, 3, 32767, 32768, 40000, 1 << 17, (1 << 20) + 3)


@pytest.mark.parametrize("cases_args", [
    {},                                                    # 60 sums: descriptors in device memory
    {"count": 20},                                         # 20 sums: descriptors in the launch parameters
    {"sizes": LARGE_SUM_SIZES, "count": 30, "seed": 9},    # large ones over the whole GPU, mixed with small
], ids=["batch", "inline", "large"])
def test_signed_sums_and_trims(hg, cases_args):
    import torch

    from hypergeometrica_gb300 import series as S

    cases = _cases(**cases_args)
    keep, rec, want = [], [], []
    for a, b, sa, sb in cases:
        ta, na = _dev(a)
        tb, nb = _dev(b)
        nout = max(na, nb) + 1 + 3
        out = torch.full((nout,), -1, dtype=torch.int64, device="cuda")
        keep += [ta, tb, out]
        rec.append([ta.data_ptr(), na, tb.data_ptr(), nb, out.data_ptr(), nout,
                    np.int64(sa).view(np.uint64), np.int64(sb).view(np.uint64)])
        want.append(sa * _as_int(a) + sb * _as_int(b))
    torch.cuda.synchronize()
    res = S._sum_records(np.array(rec, dtype=np.uint64))
    for k, (v, (sg, size)) in enumerate(zip(want, res)):
        out = keep[3 * k + 2].cpu().numpy().view(np.uint64)
        assert size == (abs(v).bit_length() + 63) // 64, k
        assert sg == (-1 if v < 0 else 1), k
        assert _as_int(out) == abs(v), k  # every limb up to nout written
    # trims of the outputs, with their written lengths
    tr = S.trim_sizes([(keep[3 * k + 2], keep[3 * k + 2].numel()) for k in range(len(cases))])
    assert list(tr) == [int(s) for _, s in res]


SERIES = {
    "chudnovsky": ("make_chudnovsky_series", O.chudnovsky_series()),
    "e": ("make_e_series", O.e_series()),
    "ramanujan": ("make_ramanujan_series", O.ramanujan_series()),
    "catalan": ("make_catalan_series", O.catalan_series()),
    "apery": ("make_apery_series", O.apery_series()),
}


@pytest.mark.parametrize("name", sorted(SERIES))
@pytest.mark.parametrize("lo,hi", [(0, 1), (0, 2), (0, 3), (0, 8), (5, 40), (0, 333)])
def test_binary_split_matches_oracle(hg, name, lo, hi):
    from hypergeometrica_gb300 import series as S

    maker, ser = SERIES[name]
    part = S.binary_split(getattr(S, maker)(), lo, hi)
    want = O.binary_split(ser, lo, hi)
    got = (part.p.to_int(), part.q.to_int(), part.b.to_int(), part.r.to_int())
    assert got == want


def test_exp_series_with_service(hg):
    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300 import series as S

    with D.Service(workspace_bytes=64 << 20, slots=2) as svc:
        part = S.binary_split(S.make_exp_series("-2/7"), 0, 150, service=svc)
        den = S.partial_denominator(part, svc)
    P, Q, B, R = O.binary_split(O.exp_series("-2/7"), 0, 150)
    assert (part.p.to_int(), part.q.to_int(), part.b.to_int(), part.r.to_int()) == (P, Q, B, R)
    assert den.to_int() == B * Q


@pytest.mark.parametrize("bits", [1 << 12, 1 << 16, 1 << 20])
def test_chudnovsky_partials_exact(hg, bits):
    """The partials mpd-pi splits for a 2^12, 2^16 and 2^20-bit pi, exactly."""
    from hypergeometrica_gb300 import series as S

    n = S.chudnovsky_terms(bits)
    part = S.binary_split(S.make_chudnovsky_series(), 0, n)
    want = O.binary_split(O.chudnovsky_series(), 0, n)
    assert (part.p.to_int(), part.q.to_int(), part.b.to_int(), part.r.to_int()) == want


@pytest.mark.parametrize("bits", [1 << 22, 1 << 24])
def test_chudnovsky_partials_residues(hg, bits):
    """The 2^22 and 2^24-bit pi partials modulo three primes."""
    from hypergeometrica_gb300 import series as S

    n = S.chudnovsky_terms(bits)
    part = S.binary_split(S.make_chudnovsky_series(), 0, n)
    vals = [x.to_int() for x in (part.p, part.q, part.b, part.r)]
    for m in ((1 << 61) - 1, 2305843009213693921, 998244353):
        assert tuple(v % m for v in vals) == O.residues(O.chudnovsky_series(), 0, n, m)
    # Q is the product of q(k) = k^3 640320^3 / 24: a check of its length too
    assert part.q.size == (vals[1].bit_length() + 63) // 64


@pytest.mark.parametrize("name", sorted(SERIES) + ["exp"])
@pytest.mark.parametrize("lo,count", [(0, 70), (10**6, 40), ((1 << 31) - 40, 40)])
def test_device_leaves_match_python(hg, name, lo, count):
    """hg_series_leaves_device against the series' own functions."""
    from hypergeometrica_gb300 import series as S

    ser = S.make_exp_series("-5/3") if name == "exp" else getattr(S, SERIES[name][0])()
    assert S._device_leaves_fit(ser, lo + count)
    limbs, ss = S._device_leaves(ser, lo, lo + count)
    host = limbs.cpu().numpy().view(np.uint64).reshape(4, count, 4)
    for i in range(count):
        k = lo + i
        pk = ser.p(k)
        for j, v in enumerate((pk, ser.q(k), ser.b(k), pk * ser.a(k))):
            size = (abs(v).bit_length() + 63) // 64
            assert ss[j, i, 1] == size and ss[j, i, 0] == (-1 if v < 0 else 1), (j, k)
            assert _as_int(host[j, i]) == abs(v), (j, k)


@pytest.mark.parametrize("name", sorted(SERIES) + ["exp"])
def test_device_nodes_match_oracle(hg, name):
    """hg_series_nodes_device: whole-node partials (one thread folding each
    range) equal the oracle's binary-split of the same ranges."""
    from hypergeometrica_gb300 import series as S

    if name == "exp":
        ser, oser = S.make_exp_series("-5/3"), O.exp_series("-5/3")
    else:
        ser, oser = getattr(S, SERIES[name][0])(), SERIES[name][1]
    ranges = [(0, 1), (0, 2), (1, 2), (0, 32), (7, 30), (1000, 1031), (10**6, 10**6 + 17),
              ((1 << 31) - 40, (1 << 31) - 8)]
    lo = np.array([r[0] for r in ranges], dtype=np.int64)
    hi = np.array([r[1] for r in ranges], dtype=np.int64)
    upper = int(hi.max())
    assert S._device_leaves_fit(ser, upper)
    limbs, ss, width = S._device_nodes(ser, lo, hi, upper)
    host = limbs.cpu().numpy().view(np.uint64).reshape(4, len(ranges), width)
    for i, (a, b) in enumerate(ranges):
        want = O.binary_split(oser, a, b)
        for j, v in enumerate(want):
            size = (abs(v).bit_length() + 63) // 64
            assert ss[j, i, 1] == size, (name, a, b, j)
            assert ss[j, i, 0] == (-1 if v < 0 else 1), (name, a, b, j)
            assert _as_int(host[j, i, :size]) == abs(v), (name, a, b, j)


def test_device_nodes_width_bound(hg):
    """A width too small for a node's values is reported as size -1; the
    kernel writes nothing past the width (checked before every write)."""
    import torch

    from hypergeometrica_gb300 import series as S
    from hypergeometrica_gb300._lib import load

    ser = S.make_chudnovsky_series()
    n, width = 2, 8
    ranges = torch.tensor([0, 1, 0, 30], dtype=torch.int64, device="cuda")
    limbs = torch.full((4 * n * width + 64,), -7, dtype=torch.int64, device="cuda")
    scratch = torch.full((2 * n * width + 64,), -7, dtype=torch.int64, device="cuda")
    ss = torch.empty(8 * n, dtype=torch.int64, device="cuda")
    st = torch.cuda.current_stream()
    assert load().hg_series_nodes_device(S._polys(ser), ranges.data_ptr(), n, width, limbs.data_ptr(),
                                         ss.data_ptr(), scratch.data_ptr(), st.cuda_stream) == 0
    out = ss.cpu().numpy().reshape(4, n, 2)
    assert (out[:, 0, 1] >= 0).all()  # one term fits
    assert (out[:, 1, 1] == -1).all()  # thirty terms do not
    assert (limbs[4 * n * width:] == -7).all() and (scratch[2 * n * width:] == -7).all()


@pytest.mark.parametrize("node_height", [0, 2, 3, 7])
def test_binary_split_node_heights(hg, monkeypatch, node_height):
    """The split's result does not depend on where the tree is cut into
    whole nodes."""
    from hypergeometrica_gb300 import series as S

    monkeypatch.setattr(S, "NODE_HEIGHT", node_height)
    for maker, oser, lo, hi in (("make_chudnovsky_series", O.chudnovsky_series(), 0, 700),
                                ("make_apery_series", O.apery_series(), 3, 260)):
        part = S.binary_split(getattr(S, maker)(), lo, hi)
        want = O.binary_split(oser, lo, hi)
        assert (part.p.to_int(), part.q.to_int(), part.b.to_int(), part.r.to_int()) == want


def test_python_leaves_for_a_series_without_polynomials(hg):
    from hypergeometrica_gb300 import series as S

    ser = S.Series(a=lambda n: 3 ** n - 7, b=lambda n: n + 2, p=lambda n: 1 if n == 0 else -(2 ** (n % 70)) - n,
                   q=lambda n: 1 if n == 0 else n * n + 1)
    assert not S._device_leaves_fit(ser, 90)
    part = S.binary_split(ser, 0, 90)
    want = O.binary_split((ser.a, ser.b, ser.p, ser.q), 0, 90)
    assert (part.p.to_int(), part.q.to_int(), part.b.to_int(), part.r.to_int()) == want


def test_small_schoolbook_batch(hg):
    """hg_mul_small_batch_device against Python integers, up to 64 x 64 limbs,
    squares and zero operands included."""
    import torch

    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300 import series as S

    rng = np.random.default_rng(17)
    xs, ys, outs, want = [], [], [], []
    for k in range(300):
        nx, ny = int(rng.integers(0, 65)), int(rng.integers(0, 65))
        a = W.limbs(3 * k + 1, nx)
        if k % 7 == 2:
            a = np.full(nx, np.uint64(2**64 - 1))
        sq = k % 5 == 0
        b = a if sq else W.limbs(3 * k + 2, ny)
        ta, _ = _dev(a)
        tb, _ = _dev(b)
        nout = a.size + b.size + (k % 3)
        o = torch.full((max(1, nout),), -1, dtype=torch.int64, device="cuda")
        xs.append((ta, a.size))
        ys.append(None if sq else (tb, b.size))
        outs.append((o, nout))
        want.append(_as_int(a) * _as_int(b))
    rec = D.product_records([t.data_ptr() for t, _ in xs], [n for _, n in xs],
                            [0 if y is None else y[0].data_ptr() for y in ys],
                            [0 if y is None else y[1] for y in ys],
                            [o.data_ptr() for o, _ in outs], [n for _, n in outs])
    torch.cuda.synchronize()
    S._multiply_records(rec, None)
    torch.cuda.synchronize()
    for k, ((o, nout), v) in enumerate(zip(outs, want)):
        got = o.cpu().numpy().view(np.uint64)[:nout]
        assert _as_int(got) == v, k
