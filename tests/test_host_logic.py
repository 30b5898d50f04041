"""Host-side logic of the package that needs no GPU."""

import numpy as np

import hypergeometrica_gb300 as H
from hypergeometrica_gb300 import mpz as M
from hypergeometrica_gb300 import workloads as W


def test_digit_round_trip():
    for n in (0, 1, 2**64 - 1, 2**64, 3**1000, 2**640):
        d = H.digits_from_int(n)
        assert H.int_from_digits(d) == n
        assert M.MPZ.from_int(-n).to_int() == -n if n else True


def test_sizes_and_bits():
    x = M.MPZ(1, np.array([5, 0, 7, 0, 0], dtype=np.uint64))
    assert M.mpz_size(x) == 3
    assert M.mpz_bit_size(x) == 64 * 2 + 3
    assert M.mpz_bit_size(M.MPZ.from_int(0)) == 0
    assert M.least_power_of_two_ge(0) == 1
    assert M.least_power_of_two_ge(4096) == 4096
    assert M.least_power_of_two_ge(4097) == 8192


def test_f_expt_matches_pow():
    for base in (3, 10, 2**64 + 1):
        for n in (0, 1, 2, 3, 17, 1000):
            assert M.f_expt(base, n, 1, lambda a, b: a * b) == base**n


def test_workload_distributions():
    u = W.limbs(1, 1000, "uniform")
    assert u[-1] != 0 and len(set(u.tolist())) == 1000
    o = W.limbs(1, 50, "ones")
    assert (o == np.uint64(2**64 - 1)).all()
    s = W.limbs(1, 100000, "sparse")
    frac = np.count_nonzero(s) / len(s)
    assert 0.005 < frac < 0.02 and s[-1] != 0
    sizes = W.log_uniform_sizes(9, 4096, 6, 14)
    assert sizes.min() >= 64 and sizes.max() <= 2**14
