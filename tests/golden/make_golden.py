"""Write tests/golden/golden.json from the pure-Python restatement.

Run from the repository root:  python tests/golden/make_golden.py

Before writing anything it checks the restatement the way the reference's own
test suite checks the Lisp (tests/ntt.lisp:121-155, tests/multiplication.lisp:
9-18, tests/mpz.lisp:25-47, tests/moduli.lisp:7-30, tests/primes.lisp:7-14):
the fast NTT against the direct DFT definition, forward/reverse inversion,
m*/fast against exact reduction, and every product against exact Python
integer multiplication.  Inputs come from SplitMix64 with fixed seeds, so the
CUDA tests can regenerate the same operands.
"""

from __future__ import annotations

import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
import restatement as R  # noqa: E402
from hypergeometrica_gb300 import workloads as W  # noqa: E402

MASK = (1 << 64) - 1


def splitmix64(seed):
    """SplitMix64 stream (Steele, Lea & Flood 2014)."""
    s = seed & MASK
    while True:
        s = (s + 0x9E3779B97F4A7C15) & MASK
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        yield z ^ (z >> 31)


def limbs(seed, n, dist="uniform"):
    """The operand generator the CUDA tests and the benchmark use."""
    return [int(v) for v in W.limbs(seed, n, dist)]


def hexl(v):
    return [format(x, "x") for x in v]


def main():
    out = {}
    moduli = R.default_moduli()
    assert moduli == [0x6280000000000001, 0x5700000000000001, 0x4180000000000001], moduli
    S = R.Scheme(moduli)
    assert S.max_trans == 55 and S.lg_modulus == 62
    gens = [R.find_finite_field_generator(m) for m in moduli]
    out["scheme"] = {
        "moduli": hexl(moduli),
        "inverses": hexl(S.inverses),
        "generators": gens,
        "max_trans": S.max_trans,
        "lg_modulus": S.lg_modulus,
        "roots": [],
        "inv_roots": [],
        "inv_lengths": [],
    }
    for power in (0, 1, 2, 6, 8, 12, 17, 25, 27, 55):
        for i in range(3):
            for kk in sorted({0, 1, power // 2, max(0, power - 1), power, 55}):
                for which in (0, 1):
                    out["scheme"]["roots"].append([power, i, kk, which, format(S.root(power, i, kk, which), "x")])
                    out["scheme"]["inv_roots"].append(
                        [power, i, kk, which, format(S.root(power, i, kk, which, inverse=True), "x")])
            for which in (0, 1):
                out["scheme"]["inv_lengths"].append([power, i, which, format(S.inv_length(power, i, which), "x")])

    # Suitable moduli for 2^53 (the listing embedded at src/moduli.lisp:213-228)
    out["suitable_2_53"] = hexl(R.find_suitable_moduli(1 << 53, 15))
    out["suitable_small"] = {str(k): hexl(R.find_suitable_moduli(1 << k, 5)) for k in (2, 5, 10, 20, 40, 55)}
    out["generator_180143985094819841"] = R.find_finite_field_generator(180143985094819841)

    # m*/fast and m*/fast2 (tests/multiplication.lisp:9-18)
    g = splitmix64(2024)
    mf, mf2 = [], []
    for i, m in enumerate(moduli):
        mi = S.inverses[i]
        pairs = [(0, 0), (m - 1, m - 1), (1, m - 1), (m - 1, 2), (m >> 1, m >> 1)]
        pairs += [(next(g) % m, next(g) % m) for _ in range(200)]
        for a, b in pairs:
            r = R.m_mul_fast(a, b, m, mi)
            assert r == a * b % m
            mf.append([i, format(a, "x"), format(b, "x"), format(r, "x")])
        for _ in range(100):
            b = next(g) % m
            a = next(g)  # Shoup accepts any 64-bit a
            bi = R.calc_b_inv(b, m)
            r = R.m_mul_fast2(b, bi, a, m)
            assert r == a * b % m
            mf2.append([i, format(b, "x"), format(bi, "x"), format(a, "x"), format(r, "x")])
    out["m_mul_fast"] = mf
    out["m_mul_fast2"] = mf2

    # Garner (tests/primes.lisp:7-14) on the scheme moduli
    gar = []
    for _ in range(50):
        n = (next(g) | (next(g) << 64) | (next(g) << 128)) % (moduli[0] * moduli[1] * moduli[2])
        vals = [n % m for m in moduli]
        mixed = R.garner(moduli, vals)
        assert R.reconstruct_from_garner(moduli, mixed) == n
        gar.append([format(n, "x"), hexl(mixed)])
    out["garner"] = gar

    # NTT spectra (tests/ntt.lisp:121-155)
    ntt = []
    for lgn in (1, 2, 6, 8, 10):
        n = 1 << lgn
        for i, m in enumerate(moduli):
            src = splitmix64(1000 * lgn + i)
            v = [next(src) % m for _ in range(n)]
            fwd = R.ntt_forward(list(v), S, i)
            w = S.root(lgn, i, 0, 0)
            if lgn <= 8:
                assert R.bit_reverse_permute(fwd) == R.ntt_forward_direct(v, m, w)
            inv = R.ntt_reverse(list(fwd), S, i)
            assert inv == v
            if lgn <= 8:
                assert R.ntt_reverse(R.bit_reverse_permute(list(v)), S, i) == R.ntt_reverse_direct(v, m, w)
            ntt.append({"lgn": lgn, "mod": i, "input": hexl(v), "forward": hexl(fwd)})
    out["ntt"] = ntt

    # Products through mpz-*/ntt and mpz-square (tests/mpz.lisp:25-47)
    prods = []
    cases = [
        (1, 1, "uniform"), (2, 2, "uniform"), (3, 1, "uniform"), (7, 5, "uniform"),
        (64, 64, "uniform"), (101, 150, "uniform"), (255, 1, "uniform"), (200, 56, "uniform"),
        (64, 64, "ones"), (100, 28, "ones"), (129, 127, "ones"), (300, 212, "sparse"), (33, 31, "sparse"),
    ]
    for idx, (nx, ny, dist) in enumerate(cases):
        x = limbs(77 + 2 * idx, nx, dist)
        y = limbs(78 + 2 * idx, ny, dist)
        res = R.mpz_mul_ntt(x, y, S)
        assert R.digits_to_int(res) == R.digits_to_int(x) * R.digits_to_int(y)
        prods.append({"kind": "mul", "dist": dist, "x": hexl(x), "y": hexl(y), "storage": hexl(res)})
    for idx, (nx, dist) in enumerate([(1, "uniform"), (5, "uniform"), (64, "uniform"), (127, "ones"),
                                      (96, "sparse")]):
        x = limbs(500 + idx, nx, dist)
        res = R.mpz_square(x, S)
        assert R.digits_to_int(res) == R.digits_to_int(x) ** 2
        prods.append({"kind": "square", "dist": dist, "x": hexl(x), "storage": hexl(res)})
    # (2^128)^2 (tests/mpz.lisp:25-30)
    x = R.int_to_digits(1 << 128)
    res = R.mpz_square(x, S)
    assert R.digits_to_int(res) == 1 << 256
    prods.append({"kind": "square", "dist": "pow2", "x": hexl(x), "storage": hexl(res)})
    out["products"] = prods

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
