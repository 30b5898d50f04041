"""mpz-expt on the GPU: the x^x^x workload of the reference's published runs.

9^(9^9) has 1,228,093,895 bits (the reference's log of that run,
logs/24apr21-999-ram.txt:224).  The device result must have exactly that
length and the residues of pow(9, 9^9, m) for independent primes m, and its
limbs must equal GMP's mpz_ui_pow_ui(9, 9^9) (a third-party exact power;
skipped where libgmp is missing).  Smaller powers are compared with
Python's exact integers.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("base,n", [(3, 1), (7, 2), (5, 123), (2**64 - 59, 1000), (12345678901234567890, 4321)])
def test_expt_device_exact(hg, base, n):
    from hypergeometrica_gb300 import series as S

    assert S.mpz_expt_device(base, n).to_int() == base**n


def test_expt_host_mirror_exact(hg):
    import hypergeometrica_gb300 as H

    for base, n in ((3, 5000), (10**40 + 7, 777)):
        assert H.mpz_expt(H.MPZ.from_int(base), n).to_int() == base**n


def test_nine_to_nine_to_nine(hg):
    from hypergeometrica_gb300 import series as S
    from hypergeometrica_gb300.mpz import int_from_digits

    x = S.mpz_expt_device(9, 9**9)
    assert x.size == -(-1228093895 // 64)
    top = int(x.t[x.size - 1].item()) & (2**64 - 1)
    assert 64 * (x.size - 1) + top.bit_length() == 1228093895
    v = int_from_digits(x.t[: x.size].cpu().numpy().view(np.uint64))
    for m in ((1 << 61) - 1, 1000000007, 2**89 - 1):
        assert v % m == pow(9, 9**9, m)


def test_nine_to_nine_to_nine_equals_gmp(hg):
    import gmp

    from hypergeometrica_gb300 import series as S

    if not gmp.available():
        pytest.skip("libgmp not installed")
    want = gmp.ui_pow_ui(9, 9**9)
    x = S.mpz_expt_device(9, 9**9)
    assert x.size == want.size
    assert np.array_equal(x.t[: x.size].cpu().numpy().view(np.uint64), want)
