"""The C oracle against the golden fixtures and the reference's embedded
known answers (CPU only)."""

import numpy as np

from conftest import h2i

# print-suitable-moduli (expt 2 53) 15, as listed in src/moduli.lisp:213-228.
SUITABLE_2_53_KAT = [
    180143985094819841, 459367161991790593, 855683929200394241, 882705526964617217, 891712726219358209,
    1261007895663738881, 1288029493427961857, 1450159080013299713, 1945555039024054273, 2053641430080946177,
    2098677426354651137, 2287828610704211969, 2422936599525326849, 2485986994308513793, 2747195772696002561,
]
# Moduli printed by the published run (logs/24apr21-999-ram.txt:199).
LOG_MODULI = [0x6280000000000001, 0x5700000000000001, 0x4180000000000001]


def test_default_moduli_match_log(oracle, golden):
    assert oracle.moduli() == LOG_MODULI
    assert h2i(golden["scheme"]["moduli"]) == LOG_MODULI


def test_suitable_moduli_kat(oracle, golden):
    buf = np.zeros(15, dtype=np.uint64)
    n = oracle.lib().hgo_find_suitable_moduli(1 << 53, 15, oracle._p(buf))
    assert n == 15
    assert [int(v) for v in buf] == SUITABLE_2_53_KAT
    assert h2i(golden["suitable_2_53"]) == SUITABLE_2_53_KAT
    for k, want in golden["suitable_small"].items():
        buf = np.zeros(5, dtype=np.uint64)
        assert oracle.lib().hgo_find_suitable_moduli(1 << int(k), 5, oracle._p(buf)) == 5
        assert [int(v) for v in buf] == h2i(want)


def test_generators(oracle, golden):
    L = oracle.lib()
    assert [L.hgo_find_generator(m) for m in LOG_MODULI] == golden["scheme"]["generators"] == [3, 5, 3]
    # src/moduli.lisp:230-231
    assert L.hgo_find_generator(180143985094819841) == 11 == golden["generator_180143985094819841"]


def test_scheme_tables(oracle, golden):
    L, s = oracle.lib(), oracle.scheme()
    sch = golden["scheme"]
    inv = [0xA655C4392D7B73A5, 0xBC52640BC52640BA, 0xFA232CF252138ABB]
    assert h2i(sch["inverses"]) == inv
    for power, i, kk, which, v in sch["roots"]:
        assert L.hgo_scheme_root(s, power, i, kk, which) == int(v, 16)
    for power, i, kk, which, v in sch["inv_roots"]:
        assert L.hgo_scheme_inv_root(s, power, i, kk, which) == int(v, 16)
    for power, i, which, v in sch["inv_lengths"]:
        assert L.hgo_scheme_inv_length(s, power, i, which) == int(v, 16)


def test_m_mul_fast_fixtures(oracle, golden):
    L = oracle.lib()
    minv = [0xA655C4392D7B73A5, 0xBC52640BC52640BA, 0xFA232CF252138ABB]
    for i, a, b, r in golden["m_mul_fast"]:
        assert L.hgo_m_mul_fast(int(a, 16), int(b, 16), LOG_MODULI[i], minv[i]) == int(r, 16)
    for i, b, bi, a, r in golden["m_mul_fast2"]:
        assert L.hgo_calc_b_inv(int(b, 16), LOG_MODULI[i]) == int(bi, 16)
        assert L.hgo_m_mul_fast2(int(b, 16), int(bi, 16), int(a, 16), LOG_MODULI[i]) == int(r, 16)


def test_ntt_fixtures(oracle, golden):
    for case in golden["ntt"]:
        v = np.array(h2i(case["input"]), dtype=np.uint64)
        fwd = oracle.ntt_forward(v, case["mod"])
        assert [int(x) for x in fwd] == h2i(case["forward"])
        assert np.array_equal(oracle.ntt_reverse(fwd, case["mod"]), v)


def test_product_fixtures(oracle, golden):
    for case in golden["products"]:
        x = np.array(h2i(case["x"]), dtype=np.uint64)
        want = h2i(case["storage"])
        if case["kind"] == "mul":
            got = oracle.mpz_mul_ntt(x, np.array(h2i(case["y"]), dtype=np.uint64))
        else:
            got = oracle.mpz_square(x)
        assert [int(v) for v in got] == want, case["kind"]


def test_num_moduli_needed(oracle):
    s = oracle.scheme()
    L = oracle.lib()
    # integer-length(N (2^64-1)^2) = 128 + lg N; three 63-bit moduli hold it up to lg N = 61
    assert L.hgo_num_moduli_needed_for_bits(s, 128 + 25) == 3
    assert L.hgo_num_moduli_needed_for_bits(s, 126) == 2
    assert L.hgo_num_moduli_needed_for_bits(s, 189) == 3
    assert L.hgo_num_moduli_needed_for_bits(s, 190) == -1
