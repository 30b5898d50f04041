"""GB300-native exact multiplication for hypergeometrica.

A CUDA (sm_103a) implementation of the reference's in-core three-prime NTT
multiplication path behind a C ABI (include/hypergeometrica_gb300.h), with a
host-side mirror of the reference's MPZ multiply interface in `mpz`.
"""

from ._lib import HGError, load  # noqa: F401
from .mpz import (  # noqa: F401
    MPZ,
    NTT_MULTIPLY_THRESHOLD,
    digits_from_int,
    f_expt,
    init,
    int_from_digits,
    mpz_expt,
    mpz_mul,
    mpz_mul_ntt,
    mpz_multiply_by_digit,
    mpz_size,
    mpz_square,
    mul_host_pipeline,
    multiply_storage_schoolboy,
    scheme_moduli,
)

__all__ = [
    "HGError",
    "MPZ",
    "NTT_MULTIPLY_THRESHOLD",
    "digits_from_int",
    "f_expt",
    "init",
    "int_from_digits",
    "load",
    "mpz_expt",
    "mpz_mul",
    "mpz_mul_ntt",
    "mpz_multiply_by_digit",
    "mpz_size",
    "mpz_square",
    "mul_host_pipeline",
    "multiply_storage_schoolboy",
    "scheme_moduli",
]
