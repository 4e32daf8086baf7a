"""GB300-native (sm_103a) Goldilocks NTT: a drop-in for the transform path of
recmo/goldilocks' `goldilocks-ntt` crate behind a C ABI (include/goldilocks_gpu.h).
"""
from .ntt import (MODULUS, GoldilocksError, Plan, bit_reverse, clear_cache, convolve, divisors, fill_uniform,
                  host_pipeline, host_pipeline_submit, intt, is_divisor, next, ntt, split, strategy, transpose)

__all__ = ["MODULUS", "GoldilocksError", "Plan", "bit_reverse", "clear_cache", "convolve", "divisors",
           "fill_uniform", "host_pipeline", "host_pipeline_submit", "intt", "is_divisor", "next", "ntt", "split", "strategy", "transpose"]
